// Residue-number-system (Chinese remainder) multi-limb GEMM on the tensor cores, for
// 256-bit operands and K up to 16384.
//
//   1. Exponents: EA_i = max_k exponent(op(A)[i,k]), EB_j likewise over op(B)[:,j].
//   2. Residues: each entry becomes the integer X = trunc(x 2^(R - E)), |X| < 2^R with
//      R = 276, and is stored as its balanced residues modulo L = 70 primes below 512
//      (fp16, exact), K contiguous.
//   3. Tensor cores (tc_gemm.cu): for each prime, S = A_l B_l^T exactly in fp32, then
//      y_l = S mod m_l.
//   4. Reconstruction: the exact sum V = sum_k X_ik X_kj satisfies
//      V / M = sum_l y_l c_l / m_l (mod 1), c_l = (M / m_l)^-1 mod m_l, with
//      |V / M| < 2^-6, so V / M is the centred fractional part of that sum, formed in
//      320-bit fixed point from the table floor(2^320 c_l / m_l); then
//      C = alpha V 2^(EA_i + EB_j - 2R) + beta C.
//
// The only rounding is the truncation of the inputs to R bits (relative 2^-276 of
// the row / column maximum) and the final conversion to 256 bits, so the error obeys
// the same normwise bound as the digit GEMM in gemm.cu.
#include <mutex>

#include "crt_tables.h"
#include "gemm.cuh"
#include "tc_gemm.cuh"

namespace sdpg {

namespace {

__constant__ int c_moduli[kCrtL];
__constant__ float c_minv[kCrtL];  // 1.0f / m_l, correctly rounded (as the division would give)
__constant__ int c_pow16[kCrtL][kCrtPowChunks];
__constant__ uint32_t c_inv[kCrtL][kCrtInvWords];
__constant__ uint32_t c_mtot[8];
__device__ int d_moduli[kCrtL];
__device__ int d_error;

struct CrtDevice {
    int *moduli = nullptr, *error = nullptr;
};

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
        CrtDevice c;
        SDPG_CUDA(cudaGetSymbolAddress((void **)&c.moduli, d_moduli));
        SDPG_CUDA(cudaGetSymbolAddress((void **)&c.error, d_error));
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
    int lg[2];   // modulus groups per entry (residue kernel)
};

template <int N>
__global__ void crt_exp_kernel(CrtOperands<N> ops, int K) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int z = blockIdx.y;
    const int op = z < ops.cnt[0] ? 0 : 1;
    const int b = op ? z - ops.cnt[0] : z;
    const int o = blockIdx.x * kExpWarps + warp;
    if (o >= ops.Opad[op]) return;
    const Operand<N> X = ops.X[op];
    int emax = INT_MIN;
    if (o < ops.O[op]) {
        const mlf<N> *base = X.X + b * X.sb + o * X.so;
        for (int k = lane; k < K; k += 32) {
            const mlf<N> *v = base + k * X.sk;
            if (v->m[N - 1] != 0) emax = max(emax, v->e);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) ops.E[op][(long long)b * ops.Opad[op] + o] = (emax == INT_MIN) ? 0 : emax;
}

// Residues of op(X)[o,k] scaled to an integer below 2^R: Q[(b L + l)][o][k], padded
// entries zero.  Threads run along k so that each modulus plane is written in
// contiguous 64-byte rows.
//
// Small operands are spread over lgroups thread groups per entry, each taking every
// lgroups-th modulus, so that enough threads are in flight.
template <int N>
__global__ void __launch_bounds__(256) crt_residue_kernel(CrtOperands<N> ops, int K, int Kpad) {
    constexpr int R = kCrtR;
    constexpr int LB = 10;
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int o = blockIdx.y * 8 + threadIdx.y;
    const int z0 = ops.cnt[0] * ops.lg[0];
    const int op = (int)blockIdx.z < z0 ? 0 : 1;
    const int zz = op ? (int)blockIdx.z - z0 : (int)blockIdx.z;
    const int lgroups = ops.lg[op];
    const int b = zz / lgroups, lg = zz - b * lgroups;
    const int O = ops.O[op], Opad = ops.Opad[op];
    const Operand<N> X = ops.X[op];
    const int *E = ops.E[op];
    __half *Q = ops.Q[op];
    if (o >= Opad || k >= Kpad) return;
    uint32_t chunk[kCrtPowChunks];
#pragma unroll
    for (int c = 0; c < kCrtPowChunks; ++c) chunk[c] = 0;
    bool neg = false;
    if (o < O && k < K) {
        const mlf<N> v = X.X[b * X.sb + o * X.so + k * X.sk];
        if (v.m[N - 1] != 0) {
            const int s = v.e - E[(long long)b * Opad + o] + R - 32 * N;  // integer = M * 2^s
            if (s > -32 * N) {
                uint32_t T[LB];
#pragma unroll
                for (int w = 0; w < LB; ++w) T[w] = (w < N) ? v.m[w] : 0u;
                if (s >= 0) {
                    ml_limb_shl<LB>(T, s >> 5);
                    ml_bit_shl<LB>(T, s & 31);
                } else {
                    ml_limb_shr<LB>(T, (-s) >> 5);
                    ml_bit_shr<LB>(T, (-s) & 31);
                }
#pragma unroll
                for (int c = 0; c < kCrtPowChunks; ++c) chunk[c] = (T[c >> 1] >> (16 * (c & 1))) & 0xFFFFu;
                neg = v.s != 0;
            }
        }
    }
    __half *q = Q + ((long long)b * kCrtL * Opad + o) * Kpad + k;
    const long long plane = (long long)Opad * Kpad;
#pragma unroll 2
    for (int l = lg; l < kCrtL; l += lgroups) {
        const int m = c_moduli[l];
        int acc = 0;  // < 18 * 65535 * 511 < 2^31
#pragma unroll
        for (int c = 0; c < kCrtPowChunks; ++c) acc += (int)chunk[c] * c_pow16[l][c];
        int r = acc - (int)((float)acc * c_minv[l]) * m;
        if (r < 0) r += m;
        if (r >= m) r -= m;
        if (2 * r > m) r -= m;  // balanced: |r| <= (m - 1) / 2
        if (neg) r = -r;
        q[l * plane] = __int2half_rn(r);
    }
}

// V / M as the centred fractional part of sum_l y_l c_l / m_l (320-bit fixed point), then
// C = alpha V 2^(EA + EB - 2R) + beta C.  Each thread takes two neighbouring outputs
// along j and reads both residues of a plane with one 32-bit load.
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

template <int N>
__global__ void __launch_bounds__(128)
    crt_reconstruct_kernel(const uint16_t *Y, int Mpad, int Npad, const int *EA, const int *EB, long long sEA,
                           long long sEB, int b0, int alpha_one, GemmProblem<N> p) {
    // outputs taken as (row, column pair) in row-major order, so narrow products
    // still fill whole warps
    const int npairs = (p.Nn + 1) >> 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)p.M * npairs) return;
    const int i = (int)(t / npairs);
    const int j = 2 * (int)(t - (long long)i * npairs);
    const int bl = blockIdx.y;
    const bool ok0 = j < p.Nn && !(p.lower_only && i < j);
    const bool ok1 = j + 1 < p.Nn && !(p.lower_only && i < j + 1);
    if (!ok0 && !ok1) return;
    const uint32_t *y = reinterpret_cast<const uint32_t *>(Y + ((long long)bl * kCrtL * Mpad + i) * Npad + j);
    const long long plane = (long long)Mpad * Npad / 2;  // in pairs
    unsigned long long a0[kCrtInvWords], a1[kCrtInvWords];
#pragma unroll
    for (int w = 0; w < kCrtInvWords; ++w) a0[w] = a1[w] = 0;
#pragma unroll 10
    for (int l = 0; l < kCrtL; ++l) {
        const uint32_t yy = __ldg(y + l * plane);
        const uint32_t y0 = yy & 0xFFFFu, y1 = yy >> 16;
#pragma unroll
        for (int w = 0; w < kCrtInvWords; ++w) {
            const uint32_t c = c_inv[l][w];
            a0[w] += (unsigned long long)y0 * c;
            a1[w] += (unsigned long long)y1 * c;
        }
    }
    const int bg = b0 + bl;
    const int ea = EA[bl * sEA + i] - 2 * kCrtR;
    if (ok0) crt_finish<N>(a0, ea + EB[bl * sEB + j], alpha_one, p, p.C + bg * p.sc + i + (long long)j * p.ldc);
    if (ok1)
        crt_finish<N>(a1, ea + EB[bl * sEB + j + 1], alpha_one, p, p.C + bg * p.sc + i + (long long)(j + 1) * p.ldc);
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

// modulus groups per entry for the residue kernel: aim at about 1200 blocks of 256
inline int residue_groups(long long blocks) {
    long long g = 1200 / (blocks > 0 ? blocks : 1);
    return (int)(g < 1 ? 1 : g > 7 ? 7 : g);
}

}  // namespace

// Longest sum the moduli cover: K 2^(2R) = 2^566 keeps |V / M| below 1/4.
constexpr int kCrtMaxK = 1 << 14;

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
                crt_exp_kernel<N><<<dim3(ceil_div(opad, kExpWarps), ops.cnt[0] + ops.cnt[1]), 32 * kExpWarps, 0, s>>>(
                    ops, p.K);
                SDPG_CHECK_LAUNCH_KTW("crt_exp_kernel", s, entries * sizeof(mlf<N>) + rows * 4);
                const int lg = residue_groups((long long)(L.Kpad / 32) * (opad / 8) * (ops.cnt[0] + ops.cnt[1]));
                ops.lg[0] = ops.lg[1] = lg;
                SDPG_KT_BEGIN(s);
                crt_residue_kernel<N><<<dim3(L.Kpad / 32, opad / 8, (ops.cnt[0] + ops.cnt[1]) * lg), dim3(32, 8), 0,
                                        s>>>(ops, p.K, L.Kpad);
                SDPG_CHECK_LAUNCH_KTW("crt_residue_kernel", s,
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
            crt_reconstruct_kernel<N><<<dim3(ceil_div((long long)p.M * ((p.Nn + 1) / 2), 128), G), 128, 0, s>>>(
                Y, L.Mpad, L.Npad, EA, EB, ab ? L.Mpad : 0, bb ? L.Npad : 0, b0, alpha_one, p);
            // every output: its kCrtL residues read, the result written, C read when beta != 0
            SDPG_CHECK_LAUNCH_KTW("crt_reconstruct_kernel", s,
                                  (double)G * p.M * p.Nn * (p.lower_only ? 0.5 : 1.0) *
                                      (2.0 * kCrtL + sizeof(mlf<N>) * (ml_is_zero(p.beta) ? 1 : 2)));
        }
    }
}

// device-wide sticky word: set by every tensor-core kernel that gave up a bounded wait
int *crt_error_word() { return crt_device().error; }

template bool crt_gemm_applies<8>(const GemmProblem<8> &);
template bool crt_gemm_applies<16>(const GemmProblem<16> &);
template size_t crt_gemm_workspace_bytes<8>(const GemmProblem<8> &);
template size_t crt_gemm_workspace_bytes<16>(const GemmProblem<16> &);
template void crt_gemm<8>(const GemmProblem<8> &, void *, cudaStream_t);
template void crt_gemm<16>(const GemmProblem<16> &, void *, cudaStream_t);

}  // namespace sdpg
