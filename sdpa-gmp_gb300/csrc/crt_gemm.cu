// Residue-number-system (Chinese remainder) multi-limb GEMM on the tensor cores, for
// 256-bit operands and K up to 16384.
//
//   1. Exponents: EA_i = max_k exponent(op(A)[i,k]), EB_j likewise over op(B)[:,j].
//   2. Residues: each entry becomes the integer X = trunc(x 2^(R - E)), |X| < 2^R with
//      R = 276, and is stored as its balanced residues modulo L = 70 primes below 512
//      (fp16, exact), K contiguous.  The residues come from the tensor cores too: with
//      X = sum_c x_c 2^(8c) (36 bytes), X mod m_l = (sum_c x_c t_lc) mod m_l where
//      t_lc = 2^(8c) mod m_l, one fp16 product of [128 entries x 64 bytes] and
//      [64 x 80 moduli] per tile, exact in fp32.
//   3. Tensor cores (tc_gemm.cu): for each prime, S = A_l B_l^T exactly in fp32, then
//      y_l = S mod m_l.
//   4. Reconstruction: the exact sum V = sum_k X_ik X_kj satisfies
//      V / M = sum_l y_l c_l / m_l (mod 1), c_l = (M / m_l)^-1 mod m_l, with
//      |V / M| < K 2^(2R) / M < 1/4 (K <= 2^14, M >= 2^568), so V / M is the centred
//      fractional part of that sum, formed in 320-bit fixed point from the table
//      floor(2^320 c_l / m_l) -- on the tensor cores as well, the table's 40 bytes per
//      modulus times the residues -- then C = alpha V 2^(EA_i + EB_j - 2R) + beta C.
//
// The only rounding is the truncation of the inputs to R bits (relative 2^-276 of
// the row / column maximum) and the final conversion to 256 bits, so the error obeys
// the same normwise bound as the digit GEMM in gemm.cu.
#include <algorithm>
#include <mutex>
#include <vector>

#include "crt_tables.h"
#include "gemm.cuh"
#include "tc_gemm.cuh"
#include "tcgen05.cuh"

namespace sdpg {

namespace {

__constant__ int c_moduli[kCrtL];
__constant__ float c_minv[kCrtL];  // 1.0f / m_l, correctly rounded (as the division would give)
__constant__ int c_pow16[kCrtL][kCrtPowChunks];
__constant__ uint32_t c_inv[kCrtL][kCrtInvWords];
__constant__ uint32_t c_mtot[8];
__constant__ uint32_t c_mdiv[kCrtL];  // ceil(2^32 / m_l): x / m_l = umulhi(x, c_mdiv[l]) for x < 2^23
__device__ int d_moduli[kCrtL];
__device__ int d_error;

// Residues on the tensor cores: an entry's integer X (below 2^276) is written as 36
// bytes x_c (X = sum_c x_c 2^(8c)); then X mod m_l = (sum_c x_c t_lc) mod m_l with
// t_lc = 2^(8c) mod m_l.  The sums are one fp16 GEMM [entries x 64 chunks] x [64 x 80
// moduli] with fp32 accumulation, exact: every partial sum is an integer below
// 36 * 255 * 508 < 2^23.
constexpr int kResChunks = 36;  // bytes of a 288-bit integer
constexpr int kResK = 64;       // GEMM K: the chunks, zero-padded (one 128-byte swizzle row)
constexpr int kResN = 80;       // GEMM N: the moduli, zero-padded to a multiple of 16
constexpr int kResM = 128;      // entries per tile (tcgen05 M)
constexpr int kResTileA = kResM * kResK * 2;  // 16 KB
constexpr int kResTileB = kResN * kResK * 2;  // 10 KB
constexpr int kResSmem = kResTileA + kResTileB + 1024 + 64;
// dynamic shared memory requested per CTA: at most four CTAs per SM, whose tensor-memory
// allocations (128 columns each) then fit the SM's 512 columns together
constexpr int kResSmemLaunch = 46 * 1024;
static_assert(kResSmem <= kResSmemLaunch, "residue kernel shared memory");
static_assert(kCrtL <= kResN && kResChunks * 8 >= kCrtR && kResChunks <= kResK, "residue GEMM shape");
static_assert((long long)kResChunks * 255 * 508 < (1 << 23), "residue sums must stay exact in fp32");

// Reconstruction on the tensor cores: with F_l = floor(2^320 c_l / m_l) written as 40 bytes
// f_lp, sum_l y_l F_l = sum_p 2^(8p) S_p where S_p = sum_l y_l f_lp: one fp16 product
// [128 outputs x 128 moduli (70 used)] x [128 x 48 bytes (40 used)] per tile with fp32
// accumulation, exact (every partial sum is an integer below 70 * 508 * 255 < 2^24).  The
// same integer as summing y_l F_l word by word, so the result is bit-identical.
constexpr int kRecBytes = 4 * kCrtInvWords;  // 40
constexpr int kRecN = 48;                    // GEMM N: the bytes, zero-padded to a multiple of 16
constexpr int kRecM = 128;                   // outputs per tile (tcgen05 M)
constexpr int kRecAtomA = kRecM * 128;       // one 64-modulus K atom of A: 16 KB
constexpr int kRecAtomB = kRecN * 128;       // one 64-modulus K atom of B: 6 KB
constexpr int kRecSmem = 2 * kRecAtomA + 2 * kRecAtomB + 1024 + 64;
// at most four CTAs per SM (tensor memory: 64 columns each would allow eight)
constexpr int kRecSmemLaunch = 52 * 1024;
static_assert(kRecSmem <= kRecSmemLaunch, "reconstruction kernel shared memory");
static_assert((long long)kCrtL * 508 * 255 < (1 << 24), "reconstruction sums must stay exact in fp32");
static_assert(kCrtL <= 128 && kRecBytes <= kRecN, "reconstruction GEMM shape");

struct CrtDevice {
    int *moduli = nullptr, *error = nullptr;
    const uint4 *rec_table = nullptr;  // f_lp as fp16: two [kRecN][64] K-major swizzled atoms (moduli 0-63, 64-127)
    const uint4 *res_table = nullptr;  // t_lc as fp16, [kResN][kResK] in the 128-byte-swizzled K-major layout
    int sms = 0;
};

// The bytes f_lp of F_l laid out as the tcgen05 B operand: atom l / 64, row p (byte), 64
// K-elements (moduli) of 2 bytes, the 16-byte chunk j of row p stored at chunk j ^ (p mod 8).
std::vector<uint16_t> reconstruct_table_host() {
    std::vector<uint16_t> t((size_t)2 * kRecN * 64, 0);
    for (int l = 0; l < kCrtL; ++l) {
        const int atom = l / 64, lk = l % 64;
        for (int pb = 0; pb < kRecBytes; ++pb) {
            const uint32_t byte = (kCrtInv[l][pb / 4] >> (8 * (pb % 4))) & 0xFFu;
            t[(size_t)atom * kRecN * 64 + (size_t)pb * 64 + (((lk / 8) ^ (pb & 7)) * 8) + lk % 8] =
                __half_as_ushort(__float2half((float)byte));  // byte < 256: exact
        }
    }
    return t;
}

// The table t_lc = 2^(8c) mod m_l laid out as the tcgen05 B operand: row l (modulus),
// 64 K-elements of 2 bytes, the 16-byte chunk j of row l stored at chunk j ^ (l mod 8).
std::vector<uint16_t> residue_table_host() {
    std::vector<uint16_t> t((size_t)kResN * kResK, 0);
    for (int l = 0; l < kCrtL; ++l) {
        const int m = kCrtModuli[l];
        int p = 1 % m;
        for (int c = 0; c < kResChunks; ++c) {
            const int j = c / 8, w = c % 8;
            t[(size_t)l * kResK + ((j ^ (l & 7)) * 8) + w] = __half_as_ushort(__float2half((float)p));  // p < 512: exact
            p = (p * 256) % m;
        }
    }
    return t;
}

// Per device: upload the tables once and look up the global-memory copies' addresses.
CrtDevice crt_device() {
    static std::mutex mu;
    static CrtDevice cache[64];
    static bool ready[64] = {};
    int dev = 0;
    SDPG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw sdpg_error(SDPG_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!ready[dev]) {
        SDPG_CUDA(cudaMemcpyToSymbol(c_moduli, kCrtModuli, sizeof(kCrtModuli)));
        float minv[kCrtL];
        for (int l = 0; l < kCrtL; ++l) minv[l] = 1.0f / (float)kCrtModuli[l];
        SDPG_CUDA(cudaMemcpyToSymbol(c_minv, minv, sizeof(minv)));
        SDPG_CUDA(cudaMemcpyToSymbol(c_pow16, kCrtPow16, sizeof(kCrtPow16)));
        SDPG_CUDA(cudaMemcpyToSymbol(c_inv, kCrtInv, sizeof(kCrtInv)));
        SDPG_CUDA(cudaMemcpyToSymbol(c_mtot, kCrtMtotMant, sizeof(kCrtMtotMant)));
        SDPG_CUDA(cudaMemcpyToSymbol(d_moduli, kCrtModuli, sizeof(kCrtModuli)));
        uint32_t mdiv[kCrtL];
        for (int l = 0; l < kCrtL; ++l)
            mdiv[l] = (uint32_t)(((1ull << 32) + (unsigned long long)kCrtModuli[l] - 1) / kCrtModuli[l]);
        SDPG_CUDA(cudaMemcpyToSymbol(c_mdiv, mdiv, sizeof(mdiv)));
        CrtDevice c;
        SDPG_CUDA(cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev));
        SDPG_CUDA(cudaGetSymbolAddress((void **)&c.moduli, d_moduli));
        SDPG_CUDA(cudaGetSymbolAddress((void **)&c.error, d_error));
        // the residue table lives for the life of the process (one per device)
        const std::vector<uint16_t> tab = residue_table_host();
        void *dt = nullptr;
        SDPG_CUDA(cudaMalloc(&dt, tab.size() * sizeof(uint16_t)));
        SDPG_CUDA(cudaMemcpy(dt, tab.data(), tab.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
        c.res_table = (const uint4 *)dt;
        const std::vector<uint16_t> rtab = reconstruct_table_host();
        void *drt = nullptr;
        SDPG_CUDA(cudaMalloc(&drt, rtab.size() * sizeof(uint16_t)));
        SDPG_CUDA(cudaMemcpy(drt, rtab.data(), rtab.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
        c.rec_table = (const uint4 *)drt;
        cache[dev] = c;
        ready[dev] = true;
    }
    return cache[dev];
}

constexpr int kExpWarps = 8;

// Both operands of a product in one launch: operand 0 is op(A) (rows i), operand 1 is
// op(B)^T (rows j); z indexes (operand, batch entry[, modulus group]).
template <int N>
struct CrtOperands {
    Operand<N> X[2];
    int O[2], Opad[2];
    int cnt[2];  // batch entries to process (0: operand not needed in this pass)
    int *E[2];
    __half *Q[2];
};

// One operand of the residue conversion: entries (o, k) of X for o < rows, k < W (W
// entries per row, rows * W a multiple of 128; a tile of 128 consecutive entries may span
// rows).  Entries with o >= O or k >= K are zero.  The
// residue of (o, k) for modulus l goes to Q[b qbatch + l qplane + o qrow + k], for rows
// o < store_rows only; the row scale is E[b ebatch + o].  With tri set, entries above the
// diagonal (o < k) count as zero.
template <int N>
struct ResSrc {
    Operand<N> X;
    int O, K, W, rows, store_rows, cnt;
    int tri;  // 1: entries with o < k are zero (the strict upper part of a lower factor)
    const int *E;
    long long ebatch;
    __half *Q;
    long long qrow, qplane, qbatch;
};

// The largest exponent of each row's nonzero entries; kExpSplit warps share a row (each
// a strided quarter of it) so that enough loads are in flight for short operands.
constexpr int kExpSplit = 4;

template <int N>
__global__ void __launch_bounds__(32 * kExpWarps) crt_exp_kernel(CrtOperands<N> ops, int K) {
    __shared__ int part[kExpWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int z = blockIdx.y;
    const int op = z < ops.cnt[0] ? 0 : 1;
    const int b = op ? z - ops.cnt[0] : z;
    const int o = blockIdx.x * (kExpWarps / kExpSplit) + warp / kExpSplit;
    const int sub = warp % kExpSplit;
    // the operand's fields are selected, not indexed by a run-time value (which would
    // put the parameter arrays in local memory)
    const int Opad = op ? ops.Opad[1] : ops.Opad[0], O = op ? ops.O[1] : ops.O[0];
    const Operand<N> X = op ? ops.X[1] : ops.X[0];
    int *E = op ? ops.E[1] : ops.E[0];
    int emax = INT_MIN;
    if (o < O) {
        const mlf<N> *base = X.X + b * X.sb + o * X.so;
        for (int k = sub * 32 + lane; k < K; k += 32 * kExpSplit) {
            const mlf<N> *v = base + k * X.sk;
            if (v->m[N - 1] != 0) emax = max(emax, v->e);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) part[warp] = emax;
    __syncthreads();
    if (sub == 0 && lane == 0 && o < Opad) {
#pragma unroll
        for (int q = 1; q < kExpSplit; ++q) emax = max(emax, part[warp + q]);
        E[(long long)b * Opad + o] = (emax == INT_MIN) ? 0 : emax;
    }
}

// Entry (o, k) of op(X) as the integer trunc(|x| 2^(R - E)) (below 2^R, R = 276) in ten
// 32-bit words, and its sign; zero for padding and for entries far below the row scale.
template <int N>
__device__ __forceinline__ bool crt_integer(const Operand<N> &X, int b, int o, int k, int O, int K, int Erow,
                                            uint32_t (&T)[10]) {
    constexpr int R = kCrtR;
#pragma unroll
    for (int w = 0; w < 10; ++w) T[w] = 0;
    if (o >= O || k >= K) return false;
    const mlf<N> v = X.X[b * X.sb + o * X.so + k * X.sk];
    if (v.m[N - 1] == 0) return false;
    const int s = v.e - Erow + R - 32 * N;  // integer = M * 2^s
    if (s <= -32 * N) return false;
#pragma unroll
    for (int w = 0; w < 10; ++w) T[w] = (w < N) ? v.m[w] : 0u;
    if (s >= 0) {
        ml_limb_shl<10>(T, s >> 5);
        ml_bit_shl<10>(T, s & 31);
    } else {
        ml_limb_shr<10>(T, (-s) >> 5);
        ml_bit_shr<10>(T, (-s) & 31);
    }
    return v.s != 0;
}

// y = s mod m_l (s < 2^23, an exact fp32 sum), balanced to |y| <= (m_l - 1) / 2, signed, as
// fp16 into residue plane L
template <int L>
__device__ __forceinline__ void store_residue(__half *q, long long plane, uint32_t bits, bool neg) {
    const uint32_t x = __float2uint_rn(__uint_as_float(bits));
    const int m = c_moduli[L];
    int r = (int)(x - __umulhi(x, c_mdiv[L]) * (uint32_t)m);
    if (2 * r > m) r -= m;
    if (neg) r = -r;
    q[(long long)L * plane] = __int2half_rn(r);
}

// columns C0 .. C0 + W - 1 of a thread's tensor-memory row: the moduli with those indices
template <int C0, int W>
struct ResidueColumns {
    template <int NR>
    static __device__ __forceinline__ void run(__half *q, long long plane, const uint32_t (&v)[NR], bool neg) {
        if constexpr (W > 0) {
            if constexpr (C0 < kCrtL) store_residue<C0>(q, plane, v[NR - W], neg);
            ResidueColumns<C0 + 1, W - 1>::run(q, plane, v, neg);
        }
    }
};

// Residues of op(X)[o, k] scaled to an integer below 2^R (ResSrc: where they go, padded
// entries zero).  A CTA takes tiles of 128 consecutive entries of the region (entry e =
// o W + k; thread t one entry): it writes the entries' 36 bytes as the rows of a
// 128 x 64 fp16 tile (128-byte swizzle), one thread issues the four K = 16 products with
// the table t_lc (80 x 64, loaded once per CTA), and each thread reduces its row of the
// 128 x 80 fp32 accumulator modulo the 70 primes.  The tile's plane stores are
// contiguous along e for every modulus.  The product wait is bounded: on time-out the
// CTA records error 4 and stops.
template <int N>
__global__ void __launch_bounds__(kResM) tc_residue_kernel(ResSrc<N> s0, ResSrc<N> s1,
                                                           const uint4 *__restrict__ table, int *error, int *sticky) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *tA = smem;
    uint8_t *tB = smem + kResTileA;
    uint64_t *bar = (uint64_t *)(tB + kResTileB);
    uint32_t *tmem_slot = (uint32_t *)(bar + 1);
    __shared__ int abort_flag;

    const int t = threadIdx.x, warp = t >> 5;
    const int z = blockIdx.y;
    const bool second = z >= s0.cnt;
    const ResSrc<N> &S = second ? s1 : s0;
    const int b = second ? z - s0.cnt : z;
    const int W = S.W, O = S.O;
    const Operand<N> X = S.X;
    const int *E = S.E + (long long)b * S.ebatch;
    const long long region = (long long)S.rows * W;
    const int ntiles = (int)(region / kResM);
    if ((int)blockIdx.x >= ntiles) return;  // the whole CTA: this operand is the smaller one

    for (int i = t; i < kResTileB / 16; i += kResM) reinterpret_cast<uint4 *>(tB)[i] = table[i];
    if (t == 0) {
        abort_flag = 0;
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(tmem_slot), 128);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    __half *qbase = S.Q + (long long)b * S.qbatch;
    const long long qplane = S.qplane;
    const __half2 k1024 = __half2half2(__ushort_as_half(0x6400));
    uint32_t phase = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, phase ^= 1u) {
        const long long e = (long long)tile * kResM + t;
        const int o = (int)(e / W), k = (int)(e - (long long)o * W);
        const int Erow = o < O ? E[o] : 0;
        uint32_t T[10];
        const bool neg = crt_integer<N>(X, b, o, k, (S.tri && o < k) ? 0 : O, S.K, Erow, T);
        // the entry's 36 bytes, each as fp16 (0x6400 | byte is 1024 + byte, minus 1024)
        uint8_t *row = tA + t * 128;
#pragma unroll
        for (int j = 0; j < kResK / 8; ++j) {  // 16-byte chunk j holds K elements 8j .. 8j + 7
            uint32_t h[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c0 = 8 * j + 2 * q, c1 = c0 + 1;
                const uint32_t b0 = c0 < kResChunks ? (T[c0 >> 2] >> (8 * (c0 & 3))) & 0xFFu : 0u;
                const uint32_t b1 = c1 < kResChunks ? (T[c1 >> 2] >> (8 * (c1 & 3))) & 0xFFu : 0u;
                const __half2 x = __halves2half2(__ushort_as_half((unsigned short)(0x6400u | b0)),
                                                 __ushort_as_half((unsigned short)(0x6400u | b1)));
                const __half2 y = __hsub2(x, k1024);
                h[q] = *reinterpret_cast<const uint32_t *>(&y);
            }
            *reinterpret_cast<uint4 *>(row + ((j ^ (t & 7)) * 16)) = make_uint4(h[0], h[1], h[2], h[3]);
        }
        // the tile was written through the generic proxy and is read by the tensor cores
        // through the async proxy; the barrier also orders the previous tile's
        // tensor-memory reads before this tile's products
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            const uint64_t ad = sw128_kmajor_desc(smem_u32(tA)), bd = sw128_kmajor_desc(smem_u32(tB));
            constexpr uint32_t idesc = idesc_f16_f32(kResM, kResN);
#pragma unroll
            for (int kk = 0; kk < kResK / 16; ++kk)
                tc_mma(tmem, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc, kk > 0 ? 1u : 0u);
            tc_commit(smem_u32(bar));
        }
        __syncwarp();
        // the products above are issued: a drain-type wait with the full budget
        if (!mbar_wait(smem_u32(bar), phase)) {
            atomicExch(error, 4);
            if (sticky && sticky != error) atomicExch(sticky, 4);
            abort_flag = 1;
        }
        __syncthreads();
        if (abort_flag) break;
        tc_fence_after();
        __half *q = qbase + (long long)o * S.qrow + k;
        const bool store = o < S.store_rows;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        uint32_t v[32];
        tmem_ld32(lane_addr, v);
        tmem_ld_wait();
        if (store) ResidueColumns<0, 32>::run(q, qplane, v, neg);
        tmem_ld32(lane_addr + 32, v);
        tmem_ld_wait();
        if (store) ResidueColumns<32, 32>::run(q, qplane, v, neg);
        uint32_t w[8];
        tmem_ld8(lane_addr + 64, w);
        tmem_ld_wait();
        if (store) ResidueColumns<64, 8>::run(q, qplane, w, neg);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

// V / M as the centred fractional part of sum_l y_l c_l / m_l (320-bit fixed point, the
// word sums acc[w] = sum_l y_l floor(2^320 c_l / m_l)[w]), then C = alpha V 2^(EA + EB - 2R)
// + beta C.
template <int N>
__device__ __forceinline__ void crt_finish(const unsigned long long (&acc)[kCrtInvWords], int escale, int alpha_one,
                                           const GemmProblem<N> &p, mlf<N> *cp) {
    uint32_t W[kCrtInvWords];
    unsigned long long carry = 0;
#pragma unroll
    for (int w = 0; w < kCrtInvWords; ++w) {
        const unsigned long long t = acc[w] + carry;
        W[w] = (uint32_t)t;
        carry = t >> 32;
    }
    // the integer part (carry out of the top word) is dropped: fractional part in [0, 1)
    const uint32_t neg = W[kCrtInvWords - 1] >> 31;
    if (neg) {  // f >= 1/2: V / M = f - 1 < 0; magnitude 2^320 - f
        unsigned long long c = 1;
#pragma unroll
        for (int w = 0; w < kCrtInvWords; ++w) {
            const unsigned long long t = (unsigned long long)(~W[w]) + c;
            W[w] = (uint32_t)t;
            c = t >> 32;
        }
    }
    const mlf<N> frac = ml_pack<N, kCrtInvWords>(W, 0, neg);  // |V| / M
    mlf<N> Mt;
    Mt.e = kCrtMtotExp;
    Mt.s = 0;
#pragma unroll
    for (int w = 0; w < N; ++w) Mt.m[w] = c_mtot[w];
    mlf<N> v = ml_ldexp(ml_mul(frac, Mt), escale);
    if (!alpha_one) v = ml_mul(v, p.alpha);
    if (!ml_is_zero(p.beta)) v = ml_add(v, ml_mul(p.beta, *cp));
    *cp = v;
}

// The reconstruction on the tensor cores.  A CTA takes tiles of 128 consecutive outputs
// (e = i Nn + j, row-major, thread t one output): each thread gathers its 70 residues
// (coalesced along j for every modulus) as one row of a 128 x 128 fp16 tile (two
// 64-modulus swizzle atoms), one thread issues the five K = 16 products with the byte
// table (48 x 128, loaded once per CTA), and each thread forms its output's 320-bit
// fixed-point sum from the 40 exact byte sums and finishes it (crt_finish).  The product
// wait is bounded: on time-out the CTA records error 5 and stops.
template <int N>
__global__ void __launch_bounds__(kRecM) tc_reconstruct_kernel(const uint16_t *Y, int Mpad, int Npad, const int *EA,
                                                               const int *EB, long long sEA, long long sEB, int b0,
                                                               int alpha_one, GemmProblem<N> p,
                                                               const uint4 *__restrict__ table, int *error,
                                                               int *sticky) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *tA = smem;                   // two atoms of 128 rows x 128 bytes
    uint8_t *tB = smem + 2 * kRecAtomA;   // two atoms of 48 rows x 128 bytes
    uint64_t *bar = (uint64_t *)(tB + 2 * kRecAtomB);
    uint32_t *tmem_slot = (uint32_t *)(bar + 1);
    __shared__ int abort_flag;
    const int t = threadIdx.x, warp = t >> 5;
    const int bl = blockIdx.y;
    const long long outputs = (long long)p.M * p.Nn;
    const int ntiles = (int)((outputs + kRecM - 1) / kRecM);
    if ((int)blockIdx.x >= ntiles) return;  // the whole CTA
    for (int q = t; q < 2 * kRecAtomB / 16; q += kRecM) reinterpret_cast<uint4 *>(tB)[q] = table[q];
    // moduli 70 .. 127 of every row stay zero: clear the second atom once
    for (int q = t; q < kRecAtomA / 16; q += kRecM) reinterpret_cast<uint4 *>(tA + kRecAtomA)[q] = make_uint4(0, 0, 0, 0);
    if (t == 0) {
        abort_flag = 0;
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(tmem_slot), 64);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const long long plane = (long long)Mpad * Npad;
    const uint16_t *ybase = Y + (long long)bl * kCrtL * plane;
    const int bg = b0 + bl;
    uint32_t phase = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, phase ^= 1u) {
        const long long e = (long long)tile * kRecM + t;
        const bool live = e < outputs;
        const int i = live ? (int)(e / p.Nn) : 0;
        const int j = live ? (int)(e - (long long)i * p.Nn) : 0;
        // the output's residues as the row t of the A tile (K element l at atom l / 64)
        const uint16_t *y = ybase + (long long)i * Npad + j;
#pragma unroll
        for (int c = 0; c < 9; ++c) {  // 16-byte chunks: moduli 8c .. 8c + 7 (chunk 8 is atom 1's first)
            uint32_t h[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int l0 = 8 * c + 2 * q, l1 = l0 + 1;
                const uint32_t v0 = (live && l0 < kCrtL) ? (uint32_t)__ldg(y + l0 * plane) : 0u;
                const uint32_t v1 = (live && l1 < kCrtL) ? (uint32_t)__ldg(y + l1 * plane) : 0u;
                const __half2 x = __halves2half2(__ushort2half_rn((unsigned short)v0), __ushort2half_rn((unsigned short)v1));
                h[q] = *reinterpret_cast<const uint32_t *>(&x);
            }
            uint8_t *row = tA + (c >> 3) * kRecAtomA + t * 128;
            const int cj = c & 7;
            *reinterpret_cast<uint4 *>(row + ((cj ^ (t & 7)) * 16)) = make_uint4(h[0], h[1], h[2], h[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            constexpr uint32_t idesc = idesc_f16_f32(kRecM, kRecN);
            const uint64_t a0 = sw128_kmajor_desc(smem_u32(tA)), b0d = sw128_kmajor_desc(smem_u32(tB));
            const uint64_t a1 = sw128_kmajor_desc(smem_u32(tA + kRecAtomA)),
                           b1d = sw128_kmajor_desc(smem_u32(tB + kRecAtomB));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                tc_mma(tmem, a0 + (uint64_t)(2 * kk), b0d + (uint64_t)(2 * kk), idesc, kk > 0 ? 1u : 0u);
            tc_mma(tmem, a1, b1d, idesc, 1u);  // moduli 64 .. 79 (70 .. 79 zero)
            tc_commit(smem_u32(bar));
        }
        __syncwarp();
        // the products above are issued: a drain-type wait with the full budget
        if (!mbar_wait(smem_u32(bar), phase)) {
            atomicExch(error, 5);
            if (sticky && sticky != error) atomicExch(sticky, 5);
            abort_flag = 1;
        }
        __syncthreads();
        if (abort_flag) break;
        tc_fence_after();
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        uint32_t v[32], w8[8];
        tmem_ld32(lane_addr, v);
        tmem_ld8(lane_addr + 32, w8);
        tmem_ld_wait();
        unsigned long long acc[kCrtInvWords];
#pragma unroll
        for (int w = 0; w < kCrtInvWords; ++w) {
            unsigned long long a = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int pb = 4 * w + q;
                const uint32_t bits = pb < 32 ? v[pb] : w8[pb - 32];
                a += (unsigned long long)__float2uint_rn(__uint_as_float(bits)) << (8 * q);
            }
            acc[w] = a;
        }
        if (live && !(p.lower_only && i < j)) {
            const int escale = EA[bl * sEA + i] - 2 * kCrtR + EB[bl * sEB + j];
            crt_finish<N>(acc, escale, alpha_one, p, p.C + bg * p.sc + i + (long long)j * p.ldc);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 64);
    }
}

template <int N>
void reconstruct_launch_tc(const uint16_t *Y, int Mpad, int Npad, const int *EA, const int *EB, long long sEA,
                           long long sEB, int b0, int alpha_one, const GemmProblem<N> &p, int batch,
                           const CrtDevice &dev, int *error, cudaStream_t s) {
    static std::once_flag once;
    std::call_once(once, [] {
        SDPG_CUDA(cudaFuncSetAttribute(tc_reconstruct_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kRecSmemLaunch));
    });
    const long long tiles = ((long long)p.M * p.Nn + kRecM - 1) / kRecM;
    const int grid_x = (int)std::min<long long>(tiles, std::max<long long>(1, 4LL * dev.sms / std::max(1, batch) + 1));
    tc_reconstruct_kernel<N><<<dim3(grid_x, batch), kRecM, kRecSmemLaunch, s>>>(
        Y, Mpad, Npad, EA, EB, sEA, sEB, b0, alpha_one, p, dev.rec_table, error ? error : dev.error, dev.error);
}

struct CrtLayout {
    int Mpad, Npad, Kpad, G, groups;
    size_t ea, eb, qa, qb, y;
    size_t total() const { return ea + eb + qa + qb + y + 6 * 256; }
};

constexpr size_t kCrtBudget = (size_t)384 << 20;  // scratch per pass; larger batches run in groups

template <int N>
CrtLayout crt_layout(const GemmProblem<N> &p) {
    CrtLayout L;
    L.Mpad = (int)round_up(p.M, kTcBM);
    L.Npad = (int)round_up(p.Nn, kTcBN);
    L.Kpad = (int)round_up(p.K, kTcBK);
    const bool ab = p.A.sb != 0, bb = p.B.sb != 0;
    const size_t qa1 = (size_t)kCrtL * L.Mpad * L.Kpad * 2, qb1 = (size_t)kCrtL * L.Npad * L.Kpad * 2;
    const size_t y1 = (size_t)kCrtL * L.Mpad * L.Npad * 2;
    const size_t per = (ab ? qa1 + L.Mpad * 4 : 0) + (bb ? qb1 + L.Npad * 4 : 0) + y1;
    const size_t fixed = (ab ? 0 : qa1 + L.Mpad * 4) + (bb ? 0 : qb1 + L.Npad * 4);
    size_t G = kCrtBudget > fixed + per ? (kCrtBudget - fixed) / per : 1;
    if (G < 1) G = 1;
    if (G > (size_t)p.batch) G = p.batch;
    L.G = (int)G;
    L.groups = (p.batch + L.G - 1) / L.G;
    L.ea = (size_t)(ab ? G : 1) * L.Mpad * 4;
    L.eb = (size_t)(bb ? G : 1) * L.Npad * 4;
    L.qa = (ab ? G : 1) * qa1;
    L.qb = (bb ? G : 1) * qb1;
    L.y = G * y1;
    return L;
}

inline char *align256(char *p) { return (char *)(((uintptr_t)p + 255) & ~(uintptr_t)255); }

// The residue conversion of up to two operands in one launch: enough CTAs to fill the SMs
// four deep, each looping over the tiles of its operand.
template <int N>
void residue_launch(const ResSrc<N> &s0, const ResSrc<N> &s1, const CrtDevice &dev, int *error, cudaStream_t s) {
    for (const ResSrc<N> *r : {&s0, &s1})
        if (r->cnt > 0 && ((long long)r->rows * r->W) % kResM != 0)
            throw sdpg_error(SDPG_ERR_ARG, "residue conversion: unsupported region shape");
    const int ops = s0.cnt + s1.cnt;
    if (ops <= 0) return;
    const long long tiles = std::max((long long)s0.rows * s0.W * (s0.cnt > 0), (long long)s1.rows * s1.W * (s1.cnt > 0)) / kResM;
    const int grid_x = (int)std::min<long long>(tiles, std::max<long long>(1, 4LL * dev.sms / ops + 1));
    tc_residue_kernel<N><<<dim3(grid_x, ops), kResM, kResSmemLaunch, s>>>(s0, s1, dev.res_table, error, dev.error);
}

}  // namespace

// Longest sum the moduli cover: K 2^(2R) = 2^566 keeps |V / M| below 1/4 (M, the product
// of the moduli, lies in [2^(kCrtMtotExp - 1), 2^kCrtMtotExp)).
constexpr int kCrtMaxK = 1 << 14;
static_assert(14 + 2 * kCrtR <= (kCrtMtotExp - 1) - 2, "K 2^(2R) / M must stay below 1/4 for K <= kCrtMaxK");

// 0: tensor-core residue path where it applies and the product is not tiny;
// 1: digit GEMM only; 2: residue path for every 256-bit product with K <= 1024
int g_gemm_method = 0;

template <int N>
bool crt_gemm_applies(const GemmProblem<N> &p) {
    if constexpr (N != 8) {
        return false;
    } else {
        if (g_gemm_method == 1 || p.K <= 0 || p.K > kCrtMaxK || p.M <= 0 || p.Nn <= 0) return false;
        return g_gemm_method == 2 || (double)p.M * p.Nn * p.K * p.batch >= (double)(1 << 15);
    }
}

template <int N>
size_t crt_gemm_workspace_bytes(const GemmProblem<N> &p) {
    return crt_layout<N>(p).total();
}

template <int N>
void crt_gemm(const GemmProblem<N> &p, void *scratch, cudaStream_t s) {
    if constexpr (N != 8) {
        throw sdpg_error(SDPG_ERR_ARG, "residue GEMM path is for 256-bit operands");
    } else {
        const CrtLayout L = crt_layout<N>(p);
        const CrtDevice dev = crt_device();
        char *cur = align256((char *)scratch);
        int *EA = (int *)cur;
        cur = align256(cur + L.ea);
        int *EB = (int *)cur;
        cur = align256(cur + L.eb);
        __half *QA = (__half *)cur;
        cur = align256(cur + L.qa);
        __half *QB = (__half *)cur;
        cur = align256(cur + L.qb);
        uint16_t *Y = (uint16_t *)cur;
        const bool ab = p.A.sb != 0, bb = p.B.sb != 0;
        const mlf<N> one = ml_one<N>();
        const int alpha_one = memcmp(&one, &p.alpha, sizeof(one)) == 0;
        for (int g = 0; g < L.groups; ++g) {
            const int b0 = g * L.G;
            const int G = min(L.G, p.batch - b0);
            const int gA = ab ? G : 1, gB = bb ? G : 1;
            CrtOperands<N> ops;
            ops.X[0] = p.A;
            ops.X[0].X += (long long)b0 * p.A.sb;
            ops.X[1] = p.B;
            ops.X[1].X += (long long)b0 * p.B.sb;
            ops.O[0] = p.M;
            ops.O[1] = p.Nn;
            ops.Opad[0] = L.Mpad;
            ops.Opad[1] = L.Npad;
            ops.cnt[0] = (g == 0 || ab) ? gA : 0;  // an operand shared by the batch is done once
            ops.cnt[1] = (g == 0 || bb) ? gB : 0;
            ops.E[0] = EA;
            ops.E[1] = EB;
            ops.Q[0] = QA;
            ops.Q[1] = QB;
            const int opad = max(L.Mpad, L.Npad);
            // algorithmic work of the conversions: every entry of the operands read once
            // (multi-limb), its kCrtL residues written once (fp16); exponents 4 bytes a row
            const double entries = ((double)ops.cnt[0] * p.M + (double)ops.cnt[1] * p.Nn) * p.K;
            const double rows = (double)ops.cnt[0] * p.M + (double)ops.cnt[1] * p.Nn;
            if (ops.cnt[0] + ops.cnt[1] > 0) {
                SDPG_KT_BEGIN(s);
                crt_exp_kernel<N><<<dim3(ceil_div(opad, kExpWarps / kExpSplit), ops.cnt[0] + ops.cnt[1]),
                                     32 * kExpWarps, 0, s>>>(ops, p.K);
                SDPG_CHECK_LAUNCH_KTW("crt_exp_kernel", s, entries * sizeof(mlf<N>) + rows * 4);
                ResSrc<N> rs[2];
                for (int q = 0; q < 2; ++q) {
                    rs[q].X = ops.X[q];
                    rs[q].O = ops.O[q];
                    rs[q].K = p.K;
                    rs[q].W = L.Kpad;
                    rs[q].rows = ops.Opad[q];
                    rs[q].store_rows = ops.Opad[q];
                    rs[q].cnt = ops.cnt[q];
                    rs[q].E = ops.E[q];
                    rs[q].ebatch = ops.Opad[q];
                    rs[q].Q = ops.Q[q];
                    rs[q].qrow = L.Kpad;
                    rs[q].qplane = (long long)ops.Opad[q] * L.Kpad;
                    rs[q].qbatch = (long long)kCrtL * ops.Opad[q] * L.Kpad;
                    rs[q].tri = 0;
                }
                SDPG_KT_BEGIN(s);
                residue_launch<N>(rs[0], rs[1], dev, p.error ? p.error : dev.error, s);
                SDPG_CHECK_LAUNCH_KTW("tc_residue_kernel", s,
                                      entries * (sizeof(mlf<N>) + 2.0 * kCrtL) + rows * 4);
            }
            TcModGemm t{};
            t.A = QA;
            t.B = QB;
            t.Y = Y;
            t.L = kCrtL;
            t.batch = G;
            t.a_batched = ab;
            t.b_batched = bb;
            t.Mpad = L.Mpad;
            t.Npad = L.Npad;
            t.kpitch = L.Kpad;
            t.lower_only = p.lower_only;
            t.moduli = dev.moduli;
            t.error = p.error ? p.error : dev.error;
            t.sticky = dev.error;
            if (p.ev_before) SDPG_CUDA(cudaEventRecord(p.ev_before, s));
            // K beyond the tensor memory's four exact accumulators runs in chunks whose
            // residues are added modulo each prime in the epilogue
            for (int k0 = 0; k0 < L.Kpad; k0 += kTcMaxK) {
                t.k0 = k0;
                t.Kpad = min(kTcMaxK, L.Kpad - k0);
                t.accumulate = k0 > 0;
                t.alg_flops = 2.0 * kCrtL * G * (double)p.M * p.Nn * min(kTcMaxK, p.K - k0) *
                              (p.lower_only ? 0.5 : 1.0);
                tc_modgemm(t, s);
            }
            if (p.ev_after) SDPG_CUDA(cudaEventRecord(p.ev_after, s));
            SDPG_KT_BEGIN(s);
            reconstruct_launch_tc<N>(Y, L.Mpad, L.Npad, EA, EB, ab ? L.Mpad : 0, bb ? L.Npad : 0, b0, alpha_one, p, G,
                                     dev, p.error, s);
            // every output: its kCrtL residues read, the result written, C read when beta != 0
            SDPG_CHECK_LAUNCH_KTW("tc_reconstruct_kernel", s,
                                  (double)G * p.M * p.Nn * (p.lower_only ? 0.5 : 1.0) *
                                      (2.0 * kCrtL + sizeof(mlf<N>) * (ml_is_zero(p.beta) ? 1 : 2)));
        }
    }
}


// ---- residues of a Cholesky factor's finished columns --------------------------------
//
// The left-looking factorisation's panel product C[k0:n, k0:k0+kb] -= L[k0:n, :k0]
// L[k0:k0+kb, :k0]^T reads every finished column again at every later panel.  With a
// row scale that does not depend on k0, the residues of a finished column stay valid,
// so each column is converted once, right after its panel is factored, into planes that
// every later panel product reads directly.  The scale of row i is 2^E_i with
// E_i = ceil(e_i / 2) + 1, A_ii in [2^(e_i - 1), 2^e_i): |L_ik| <= sqrt(A_ii) < 2^(E_i - 1)
// for a positive definite A, so every integer stays below 2^R.  The truncation error of a
// product entry is then at most K 2^(E_i + E_j - R), the form of Cholesky's own backward
// error bound (|L| |L|^T <= sqrt(A_ii A_jj) entrywise).

namespace {

template <int N>
__global__ void cache_scale_kernel(int n, const mlf<N> *A, long long lda, int *E) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const mlf<N> d = A[i + (long long)i * lda];
    // ceil(e / 2) for either sign of e, plus the margin bit
    E[i] = (ml_is_zero(d) ? 0 : (d.e >= 0 ? (d.e + 1) / 2 : -((-d.e) / 2))) + 1;
}

}  // namespace

size_t crt_cache_bytes(int n) {
    const size_t rows = round_up(n, kTcBM), kp = round_up(n, kTcBK);
    const size_t planes = (size_t)kCrtL * rows * kp * 2;
    const size_t y = (size_t)kCrtL * rows * kTcBN * 2;  // one panel product's result planes
    return planes + y + rows * 4 + 4 * 256;
}

template <int N>
bool crt_cache_applies(int n) {
    if constexpr (N != 8) {
        return false;
    } else {
        return g_gemm_method != 1 && n >= kTcBM && n <= kCrtMaxK;
    }
}

template <int N>
CrtCache crt_cache_init(int n, const mlf<N> *A, long long lda, void *mem, cudaStream_t s) {
    CrtCache c;
    c.n = n;
    c.rows = (int)round_up(n, kTcBM);
    c.kpitch = (int)round_up(n, kTcBK);
    char *cur = align256((char *)mem);
    c.Q = (__half *)cur;
    cur = align256(cur + (size_t)kCrtL * c.rows * c.kpitch * 2);
    c.Y = (uint16_t *)cur;
    cur = align256(cur + (size_t)kCrtL * c.rows * kTcBN * 2);
    c.E = (int *)cur;
    // planes start at zero: columns not yet finished and the upper triangle read as zero
    SDPG_CUDA(cudaMemsetAsync(c.Q, 0, (size_t)kCrtL * c.rows * c.kpitch * 2, s));
    SDPG_KT_BEGIN(s);
    cache_scale_kernel<N><<<ceil_div(n, 128), 128, 0, s>>>(n, A, lda, c.E);
    SDPG_CHECK_LAUNCH_KT("cache_scale_kernel", s);
    return c;
}

template <int N>
void crt_cache_put(const CrtCache &c, const mlf<N> *A, long long lda, int k0, int kb, int *error, cudaStream_t s) {
    if constexpr (N != 8) {
        throw sdpg_error(SDPG_ERR_ARG, "residue path is for 256-bit operands");
    } else {
        const CrtDevice dev = crt_device();
        const int rows = c.n - k0;
        ResSrc<N> r{};
        r.X = Operand<N>{A + k0 + (long long)k0 * lda, 1, lda, 0};
        r.O = rows;
        r.K = kb;
        r.W = 32;
        r.rows = (int)round_up(rows, kResM / 32);
        r.store_rows = rows;
        r.cnt = 1;
        r.tri = 1;
        r.E = c.E + k0;
        r.ebatch = 0;
        r.Q = c.Q + (long long)k0 * c.kpitch + k0;
        r.qrow = c.kpitch;
        r.qplane = (long long)c.rows * c.kpitch;
        r.qbatch = 0;
        ResSrc<N> none{};
        SDPG_KT_BEGIN(s);
        residue_launch<N>(r, none, dev, error ? error : dev.error, s);
        SDPG_CHECK_LAUNCH_KTW("tc_residue_kernel", s, (double)rows * kb * (sizeof(mlf<N>) + 2.0 * kCrtL));
    }
}

template <int N>
void crt_cache_panel(const CrtCache &c, int k0, int kb, int kend, mlf<N> *A, long long lda, int *error,
                     cudaStream_t s) {
    if constexpr (N != 8) {
        throw sdpg_error(SDPG_ERR_ARG, "residue path is for 256-bit operands");
    } else {
        const CrtDevice dev = crt_device();
        const int M = c.n - k0;
        TcModGemm t{};
        t.A = c.Q + (long long)k0 * c.kpitch;
        t.B = t.A;
        t.Y = c.Y;
        t.L = kCrtL;
        t.batch = 1;
        t.Mpad = (int)round_up(M, kTcBM);
        t.Npad = kTcBN;
        t.a_rows = t.b_rows = c.rows;
        t.a_skip = t.b_skip = k0;
        t.kpitch = c.kpitch;
        t.kext = kend;  // columns from kend on (not yet in the cache, or applied elsewhere) read as zero
        t.lower_only = 1;
        t.moduli = dev.moduli;
        t.error = error ? error : dev.error;
        t.sticky = dev.error;
        const int Kpad = (int)round_up(kend, kTcBK);
        for (int q0 = 0; q0 < Kpad; q0 += kTcMaxK) {
            t.k0 = q0;
            t.Kpad = std::min(kTcMaxK, Kpad - q0);
            t.accumulate = q0 > 0;
            t.alg_flops = 2.0 * kCrtL * (double)M * kb * std::min(kTcMaxK, kend - q0);
            tc_modgemm(t, s);
        }
        GemmProblem<N> p{};
        p.M = M;
        p.Nn = kb;
        p.K = kend;
        p.batch = 1;
        p.C = A + k0 + (long long)k0 * lda;
        p.ldc = lda;
        p.sc = 0;
        p.alpha = ml_from_int<N>(-1);
        p.beta = ml_one<N>();
        p.lower_only = 1;
        SDPG_KT_BEGIN(s);
        reconstruct_launch_tc<N>(c.Y, t.Mpad, t.Npad, c.E + k0, c.E + k0, 0, 0, 0, 0, p, 1, dev, error, s);
        SDPG_CHECK_LAUNCH_KTW("tc_reconstruct_kernel", s,
                              (double)M * kb * (2.0 * kCrtL + 2.0 * sizeof(mlf<N>)));
    }
}

template bool crt_cache_applies<8>(int);
template bool crt_cache_applies<16>(int);
template CrtCache crt_cache_init<8>(int, const mlf<8> *, long long, void *, cudaStream_t);
template CrtCache crt_cache_init<16>(int, const mlf<16> *, long long, void *, cudaStream_t);
template void crt_cache_put<8>(const CrtCache &, const mlf<8> *, long long, int, int, int *, cudaStream_t);
template void crt_cache_put<16>(const CrtCache &, const mlf<16> *, long long, int, int, int *, cudaStream_t);
template void crt_cache_panel<8>(const CrtCache &, int, int, int, mlf<8> *, long long, int *, cudaStream_t);
template void crt_cache_panel<16>(const CrtCache &, int, int, int, mlf<16> *, long long, int *, cudaStream_t);

// device-wide sticky word: set by every tensor-core kernel that gave up a bounded wait
int *crt_error_word() { return crt_device().error; }

template bool crt_gemm_applies<8>(const GemmProblem<8> &);
template bool crt_gemm_applies<16>(const GemmProblem<16> &);
template size_t crt_gemm_workspace_bytes<8>(const GemmProblem<8> &);
template size_t crt_gemm_workspace_bytes<16>(const GemmProblem<16> &);
template void crt_gemm<8>(const GemmProblem<8> &, void *, cudaStream_t);
template void crt_gemm<16>(const GemmProblem<16> &, void *, cudaStream_t);

}  // namespace sdpg
