// Block-floating-point multi-limb GEMM kernels; see gemm.cuh for the method.
#include <limits.h>

#include "gemm.cuh"

namespace sdpg {

namespace {

constexpr int kQuantWarps = 8;

// Per-outer-index shared exponent: EA[b][o] = max_k exponent(op(X)[o,k]).
template <int N>
__global__ void bfp_exp_kernel(Operand<N> X, int O, int K, int Opad, int *E) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int o = blockIdx.x * kQuantWarps + warp;
    const int b = blockIdx.y;
    if (o >= Opad) return;
    int emax = INT_MIN;
    if (o < O) {
        const mlf<N> *base = X.X + b * X.sb + o * X.so;
        for (int k = lane; k < K; k += 32) {
            const mlf<N> *v = base + k * X.sk;
            if (v->m[N - 1] != 0) emax = max(emax, v->e);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) E[(long long)b * Opad + o] = (emax == INT_MIN) ? 0 : emax;
}

// Digits of op(X)[o,k] scaled by 2^(R - E[o]); planes Q[b][d][k][o] over the padded range.
template <int N>
__global__ void bfp_digits_kernel(Operand<N> X, int O, int K, int Opad, int Kpad, const int *E, int *Q) {
    constexpr int D = Bfp<N>::D;
    constexpr int R = Bfp<N>::R;
    constexpr int LB = ((28 * D + 31) / 32 > N ? (28 * D + 31) / 32 : N) + 2;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (o >= Opad || k >= Kpad) return;
    int dig[D];
#pragma unroll
    for (int t = 0; t < D; ++t) dig[t] = 0;
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
                for (int t = 0; t < D; ++t) {
                    const int bit = 28 * t;
                    const int w = bit >> 5, r = bit & 31;
                    uint32_t lo = T[w] >> r;
                    uint32_t hi = (r > 4 && w + 1 < LB) ? (T[w + 1] << (32 - r)) : 0u;
                    dig[t] = (int)((lo | hi) & 0x0FFFFFFFu);
                }
                // balance: digits into [-2^27, 2^27)
#pragma unroll
                for (int t = 0; t < D - 1; ++t) {
                    if (dig[t] >= (1 << 27)) {
                        dig[t] -= (1 << 28);
                        dig[t + 1] += 1;
                    }
                }
                if (v.s) {
#pragma unroll
                    for (int t = 0; t < D; ++t) dig[t] = -dig[t];
                }
            }
        }
    }
    int *q = Q + (long long)b * D * Kpad * Opad + (long long)k * Opad + o;
#pragma unroll
    for (int t = 0; t < D; ++t) q[(long long)t * Kpad * Opad] = dig[t];
}

template <int NC>
__device__ __forceinline__ void carry_normalise(long long (&acc)[NC]) {
#pragma unroll
    for (int c = 0; c < NC - 1; ++c) {
        const long long carry = acc[c] >> 28;
        acc[c] -= carry << 28;
        acc[c + 1] += carry;
    }
}

// Integer columns (acc[0] at weight 2^(28*C0)) -> mlf, value * 2^(escale).
template <int N, int NC>
__device__ __forceinline__ mlf<N> columns_to_mlf(long long (&acc)[NC], int escale) {
    carry_normalise<NC>(acc);
    uint32_t sign = 0;
    if (acc[NC - 1] < 0) {
        sign = 1;
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = -acc[c];
        carry_normalise<NC>(acc);
    }
    constexpr int LW = (28 * NC + 31) / 32 + 1;
    uint32_t W[LW];
#pragma unroll
    for (int w = 0; w < LW; ++w) W[w] = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int bit = 28 * c;
        const int w = bit >> 5, r = bit & 31;
        const unsigned long long d = (unsigned long long)acc[c];  // < 2^28 except the top column
        W[w] |= (uint32_t)(d << r);
        if (w + 1 < LW) W[w + 1] |= (uint32_t)(d >> (32 - r));
        if (w + 2 < LW && r > 0) W[w + 2] |= (uint32_t)((d >> (32 - r)) >> 32);
    }
    return ml_pack<N, LW>(W, 32 * LW + escale, sign);
}

template <int N, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), 2)
bfp_gemm_kernel(const int *__restrict__ Aq, const int *__restrict__ Bq, const int *__restrict__ EA,
                const int *__restrict__ EB, int Mpad, int Npad, int Kpad, long long sAq, long long sBq,
                long long sEA, long long sEB, int alpha_one, GemmProblem<N> p) {
    constexpr int D = Bfp<N>::D;
    constexpr int NC = Bfp<N>::NC;
    constexpr int C0 = Bfp<N>::C0;
    constexpr int CH = Bfp<N>::CH;
    constexpr int TX = BN / TN;  // threads along j
    constexpr int TY = BM / TM;  // threads along i
    constexpr int NT = TX * TY;
    __shared__ __align__(16) int As[D][BK][BM];
    __shared__ __align__(16) int Bs[D][BK][BN];

    const int b = blockIdx.z;
    const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
    if (p.lower_only && i0 + BM - 1 < j0) return;  // tile strictly above the diagonal
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int *Ab = Aq + b * sAq;
    const int *Bb = Bq + b * sBq;

    long long acc[TM][TN][NC];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int c = 0; c < TN; ++c)
#pragma unroll
            for (int t = 0; t < NC; ++t) acc[a][c][t] = 0;

    int since = 0;
    for (int k0 = 0; k0 < Kpad; k0 += BK) {
        // stage digits: rows (d, kk) of BM (BN) contiguous ints
        for (int idx = threadIdx.x; idx < D * BK * (BM / 4); idx += NT) {
            const int c4 = idx % (BM / 4), row = idx / (BM / 4);
            const int d = row / BK, kk = row % BK;
            const int4 v = *reinterpret_cast<const int4 *>(Ab + ((long long)d * Kpad + k0 + kk) * Mpad + i0 + 4 * c4);
            *reinterpret_cast<int4 *>(&As[d][kk][4 * c4]) = v;
        }
        for (int idx = threadIdx.x; idx < D * BK * (BN / 4); idx += NT) {
            const int c4 = idx % (BN / 4), row = idx / (BN / 4);
            const int d = row / BK, kk = row % BK;
            const int4 v = *reinterpret_cast<const int4 *>(Bb + ((long long)d * Kpad + k0 + kk) * Npad + j0 + 4 * c4);
            *reinterpret_cast<int4 *>(&Bs[d][kk][4 * c4]) = v;
        }
        __syncthreads();
#pragma unroll 1
        for (int kk = 0; kk < BK; ++kk) {
            int av[TM][D], bv[TN][D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
#pragma unroll
                for (int a = 0; a < TM; ++a) av[a][d] = As[d][kk][ty * TM + a];
#pragma unroll
                for (int c = 0; c < TN; ++c) bv[c][d] = Bs[d][kk][tx * TN + c];
            }
            // digit-pair order: consecutive multiply-adds go to different column
            // accumulators (and different outputs), so no two back-to-back IMAD.WIDE
            // depend on each other
#pragma unroll
            for (int pp = 0; pp < D; ++pp)
#pragma unroll
                for (int qq = 0; qq < D; ++qq) {
                    if (pp + qq < C0) continue;
#pragma unroll
                    for (int a = 0; a < TM; ++a)
#pragma unroll
                        for (int c = 0; c < TN; ++c)
                            acc[a][c][pp + qq - C0] += (long long)av[a][pp] * (long long)bv[c][qq];
                }
        }
        since += BK;
        if (since >= CH) {
            since = 0;
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int c = 0; c < TN; ++c) carry_normalise<NC>(acc[a][c]);
        }
        __syncthreads();
    }

    // epilogue
    constexpr int R = Bfp<N>::R;
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        const int i = i0 + ty * TM + a;
#pragma unroll
        for (int c = 0; c < TN; ++c) {
            const int j = j0 + tx * TN + c;
            if (i >= p.M || j >= p.Nn) continue;
            if (p.lower_only && i < j) continue;
            const int escale = 28 * C0 + EA[b * sEA + i] + EB[b * sEB + j] - 2 * R;
            mlf<N> v = columns_to_mlf<N, NC>(acc[a][c], escale);
            if (!alpha_one) v = ml_mul(v, p.alpha);
            mlf<N> *cp = p.C + b * p.sc + i + (long long)j * p.ldc;
            if (!ml_is_zero(p.beta)) v = ml_add(v, ml_mul(p.beta, *cp));
            *cp = v;
        }
    }
}

template <int N>
struct GemmTiles;
template <>
struct GemmTiles<8> {
    static constexpr int BM = 32, BN = 32, BK = 16, TM = 2, TN = 2;
};
template <>
struct GemmTiles<16> {
    static constexpr int BM = 32, BN = 16, BK = 8, TM = 2, TN = 1;
};

template <int N>
struct GemmLayout {
    int Mpad, Npad, Kpad;
    size_t a_bytes, b_bytes, ea_bytes, eb_bytes;
    int batchA, batchB;
    size_t total() const { return a_bytes + b_bytes + ea_bytes + eb_bytes + 4 * 256; }
};

template <int N>
GemmLayout<N> gemm_layout(const GemmProblem<N> &p) {
    using T = GemmTiles<N>;
    constexpr int D = Bfp<N>::D;
    GemmLayout<N> L;
    L.Mpad = (int)round_up(p.M, T::BM);
    L.Npad = (int)round_up(p.Nn, T::BN);
    L.Kpad = (int)round_up(p.K > 0 ? p.K : 1, T::BK);
    L.batchA = p.A.sb == 0 ? 1 : p.batch;
    L.batchB = p.B.sb == 0 ? 1 : p.batch;
    L.a_bytes = (size_t)L.batchA * D * L.Kpad * L.Mpad * sizeof(int);
    L.b_bytes = (size_t)L.batchB * D * L.Kpad * L.Npad * sizeof(int);
    L.ea_bytes = (size_t)L.batchA * L.Mpad * sizeof(int);
    L.eb_bytes = (size_t)L.batchB * L.Npad * sizeof(int);
    return L;
}

inline char *align256(char *p) { return (char *)(((uintptr_t)p + 255) & ~(uintptr_t)255); }

}  // namespace

template <int N>
size_t gemm_bfp_workspace_bytes(const GemmProblem<N> &p) {
    return gemm_layout<N>(p).total();
}

template <int N>
size_t gemm_workspace_bytes(const GemmProblem<N> &p) {
    return crt_gemm_applies<N>(p) ? crt_gemm_workspace_bytes<N>(p) : gemm_bfp_workspace_bytes<N>(p);
}

template <int N>
void ml_gemm_scratch(const GemmProblem<N> &p, void *scratch, cudaStream_t stream) {
    using T = GemmTiles<N>;
    if (p.M <= 0 || p.Nn <= 0 || p.batch <= 0) return;
    const GemmLayout<N> L = gemm_layout<N>(p);
    char *cur = align256((char *)scratch);
    int *Aq = (int *)cur;
    cur = align256(cur + L.a_bytes);
    int *Bq = (int *)cur;
    cur = align256(cur + L.b_bytes);
    int *EA = (int *)cur;
    cur = align256(cur + L.ea_bytes);
    int *EB = (int *)cur;
    // exponents
    {
        dim3 g(ceil_div(L.Mpad, kQuantWarps), L.batchA);
        SDPG_KT_BEGIN(stream);
        bfp_exp_kernel<N><<<g, 32 * kQuantWarps, 0, stream>>>(p.A, p.M, p.K, L.Mpad, EA);
        SDPG_CHECK_LAUNCH_KT("bfp_exp_kernel", stream);
        dim3 g2(ceil_div(L.Npad, kQuantWarps), L.batchB);
        SDPG_KT_BEGIN(stream);
        bfp_exp_kernel<N><<<g2, 32 * kQuantWarps, 0, stream>>>(p.B, p.Nn, p.K, L.Npad, EB);
        SDPG_CHECK_LAUNCH_KT("bfp_exp_kernel", stream);
    }
    // digits
    {
        dim3 blk(32, 8);
        dim3 g(ceil_div(L.Mpad, 32), ceil_div(L.Kpad, 8), L.batchA);
        SDPG_KT_BEGIN(stream);
        bfp_digits_kernel<N><<<g, blk, 0, stream>>>(p.A, p.M, p.K, L.Mpad, L.Kpad, EA, Aq);
        SDPG_CHECK_LAUNCH_KT("bfp_digits_kernel", stream);
        dim3 g2(ceil_div(L.Npad, 32), ceil_div(L.Kpad, 8), L.batchB);
        SDPG_KT_BEGIN(stream);
        bfp_digits_kernel<N><<<g2, blk, 0, stream>>>(p.B, p.Nn, p.K, L.Npad, L.Kpad, EB, Bq);
        SDPG_CHECK_LAUNCH_KT("bfp_digits_kernel", stream);
    }
    constexpr int D = Bfp<N>::D;
    const long long sAq = (p.A.sb == 0) ? 0 : (long long)D * L.Kpad * L.Mpad;
    const long long sBq = (p.B.sb == 0) ? 0 : (long long)D * L.Kpad * L.Npad;
    const long long sEA = (p.A.sb == 0) ? 0 : L.Mpad;
    const long long sEB = (p.B.sb == 0) ? 0 : L.Npad;
    dim3 grid(L.Npad / T::BN, L.Mpad / T::BM, p.batch);
    constexpr int threads = (T::BM / T::TM) * (T::BN / T::TN);
    const mlf<N> one = ml_one<N>();
    const int alpha_one = memcmp(&one, &p.alpha, sizeof(one)) == 0;
    if (p.ev_before) SDPG_CUDA(cudaEventRecord(p.ev_before, stream));
    SDPG_KT_BEGIN(stream);
    bfp_gemm_kernel<N, T::BM, T::BN, T::BK, T::TM, T::TN><<<grid, threads, 0, stream>>>(
        Aq, Bq, EA, EB, L.Mpad, L.Npad, L.Kpad, sAq, sBq, sEA, sEB, alpha_one, p);
    SDPG_CHECK_LAUNCH_KT("bfp_gemm_kernel", stream);
    if (p.ev_after) SDPG_CUDA(cudaEventRecord(p.ev_after, stream));
}

template <int N>
void ml_gemm(const GemmProblem<N> &p, Workspace &ws, cudaStream_t stream) {
    if (p.M <= 0 || p.Nn <= 0 || p.batch <= 0) return;
    if (crt_gemm_applies<N>(p)) {
        void *s = ws.carve(crt_gemm_workspace_bytes<N>(p));
        if (!p.error && ws.error) {
            GemmProblem<N> q = p;
            q.error = ws.error;
            crt_gemm<N>(q, s, stream);
        } else {
            crt_gemm<N>(p, s, stream);
        }
        return;
    }
    void *s = ws.carve(gemm_bfp_workspace_bytes<N>(p));
    ml_gemm_scratch(p, s, stream);
}

#define SDPG_INST_GEMM(N)                                                                  \
    template size_t gemm_workspace_bytes<N>(const GemmProblem<N> &);                        \
    template size_t gemm_bfp_workspace_bytes<N>(const GemmProblem<N> &);                    \
    template void ml_gemm_scratch<N>(const GemmProblem<N> &, void *, cudaStream_t);        \
    template void ml_gemm<N>(const GemmProblem<N> &, Workspace &, cudaStream_t);
SDPG_INST_GEMM(8)
SDPG_INST_GEMM(16)

}  // namespace sdpg
