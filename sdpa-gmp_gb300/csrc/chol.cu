// Cholesky factorisation, triangular inverse and triangular solves in
// multi-limb arithmetic (replacing Rpotrf / Rtrsm / Rtrsv as called from
// Lal::choleskyFactorWithAdjust, Lal::getCholesky, Lal::getInvLowTriangularMatrix
// and Lal::solveSystems, sdpa_linear.cpp:342-455, 608-695).
//
// Blocked right-looking with 32-wide panels: the diagonal block is factored in
// one CTA (pivot square roots and reciprocals in full multi-limb precision), the
// panel below is solved one row per warp, and the trailing matrix is updated by
// the block-floating-point GEMM (lower triangle only).
#include "kernels.cuh"
#include "mlwarp.cuh"

namespace sdpg {

namespace {

constexpr int NB = 32;

// Factor the kb x kb diagonal block at A (ld lda) in place; rinv[j] = 1/L[j][j].
// info: 0, or (col0 + j + 1) for the first non-positive pivot.
template <int N>
__global__ void potf2_kernel(mlf<N> *A, int lda, int kb, int col0, int *info, mlf<N> *rinv) {
    __shared__ int bad;
    if (*info != 0) return;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (threadIdx.x == 0) {
            const mlf<N> d = A[j + (long long)j * lda];
            if (ml_sign(d) <= 0) {
                bad = col0 + j + 1;
            } else {
                const mlf<N> r = ml_rsqrt(d);
                A[j + (long long)j * lda] = ml_mul(d, r);  // sqrt(d)
                rinv[j] = r;
            }
        }
        __syncthreads();
        if (bad) break;
        const mlf<N> r = rinv[j];
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x)
            A[i + (long long)j * lda] = ml_mul(A[i + (long long)j * lda], r);
        __syncthreads();
        // trailing lower triangle of the block: A[i,t] -= L[i,j] L[t,j], j < t <= i < kb
        const int w = kb - j - 1;
        const int cnt = w * (w + 1) / 2;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            // q -> (ii, tt) with 0 <= tt <= ii < w
            int ii = (int)((sqrtf(8.0f * q + 1.0f) - 1.0f) * 0.5f);
            while (ii * (ii + 1) / 2 > q) --ii;
            while ((ii + 1) * (ii + 2) / 2 <= q) ++ii;
            const int tt = q - ii * (ii + 1) / 2;
            const int i = j + 1 + ii, t = j + 1 + tt;
            mlf<N> *a = A + i + (long long)t * lda;
            *a = ml_sub(*a, ml_mul(A[i + (long long)j * lda], A[t + (long long)j * lda]));
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && bad) *info = bad;
}

// Rows below the diagonal block: solve x * L11^T = a for each row (one warp per row).
// L11 at Ld (ld lda, kb x kb lower), rows at R (ld lda), nrows rows.
template <int N>
__global__ void panel_trsm_kernel(const mlf<N> *Ld, mlf<N> *R, int lda, int kb, int nrows, const int *info,
                                  const mlf<N> *rinv) {
    if (*info != 0) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    mlf<N> *row = R + warp;  // element t at row[t * lda]
    mlf<N> a = lane < kb ? row[(long long)lane * lda] : ml_zero<N>();
    for (int j = 0; j < kb; ++j) {
        mlf<N> xj = ml_zero<N>();
        if (lane == j) xj = ml_mul(a, rinv[j]);
        xj = ml_shfl(xj, j);
        if (lane == j) a = xj;
        if (lane > j && lane < kb) a = ml_sub(a, ml_mul(xj, Ld[lane + (long long)j * lda]));
    }
    if (lane < kb) row[(long long)lane * lda] = a;
}

// Invert every kb x kb diagonal block of the lower-triangular L into Linv.
template <int N>
__global__ void trtri_diag_kernel(const mlf<N> *L, int ldl, mlf<N> *Linv, int ldi, int n) {
    const int b = blockIdx.x;
    const int o = b * NB;
    const int kb = min(NB, n - o);
    const mlf<N> *T = L + o + (long long)o * ldl;
    mlf<N> *X = Linv + o + (long long)o * ldi;
    __shared__ mlf<N> rv[NB];
    if (threadIdx.x < kb) rv[threadIdx.x] = ml_recip(T[threadIdx.x + (long long)threadIdx.x * ldl]);
    // X = I (lower part)
    for (int q = threadIdx.x; q < kb * kb; q += blockDim.x) {
        const int i = q % kb, c = q / kb;
        if (i >= c) X[i + (long long)c * ldi] = (i == c) ? ml_one<N>() : ml_zero<N>();
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        // row j of X scaled by 1/T[j,j] (columns c <= j)
        for (int c = threadIdx.x; c <= j; c += blockDim.x) X[j + (long long)c * ldi] = ml_mul(X[j + (long long)c * ldi], rv[j]);
        __syncthreads();
        // X[i,c] -= T[i,j] X[j,c] for i > j, c <= j
        const int rows = kb - j - 1, cols = j + 1;
        for (int q = threadIdx.x; q < rows * cols; q += blockDim.x) {
            const int i = j + 1 + q % rows, c = q / rows;
            mlf<N> *x = X + i + (long long)c * ldi;
            *x = ml_sub(*x, ml_mul(T[i + (long long)j * ldl], X[j + (long long)c * ldi]));
        }
        __syncthreads();
    }
}

// Inverses of the NB x NB diagonal blocks of the lower-triangular L, packed:
// Dinv[b] (ld NB, lower, zeros above) = L[bNB:, bNB:]^{-1} restricted to the block.
template <int N>
__global__ void trtri_diag_packed_kernel(const mlf<N> *L, int ldl, mlf<N> *Dinv, int n) {
    const int b = blockIdx.x;
    const int o = b * NB;
    const int kb = min(NB, n - o);
    const mlf<N> *T = L + o + (long long)o * ldl;
    mlf<N> *X = Dinv + (long long)b * NB * NB;
    __shared__ mlf<N> rv[NB];
    if (threadIdx.x < kb) rv[threadIdx.x] = ml_recip(T[threadIdx.x + (long long)threadIdx.x * ldl]);
    for (int q = threadIdx.x; q < NB * NB; q += blockDim.x) {
        const int i = q % NB, c = q / NB;
        X[i + NB * c] = (i == c && i < kb) ? ml_one<N>() : ml_zero<N>();
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        for (int c = threadIdx.x; c <= j; c += blockDim.x) X[j + NB * c] = ml_mul(X[j + NB * c], rv[j]);
        __syncthreads();
        const int rows = kb - j - 1, cols = j + 1;
        for (int q = threadIdx.x; q < rows * cols; q += blockDim.x) {
            const int i = j + 1 + q % rows, c = q / rows;
            mlf<N> *x = X + i + NB * c;
            *x = ml_sub(*x, ml_mul(T[i + (long long)j * ldl], X[j + NB * c]));
        }
        __syncthreads();
    }
}

// sum_{j<cnt} a[j*stride] * y[j] with four independent accumulator chains
template <int N>
__device__ __forceinline__ mlf<N> dot_ld(const mlf<N> *a, long long stride, const mlf<N> *y, int cnt) {
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>(), a2 = ml_zero<N>(), a3 = ml_zero<N>();
    int j = 0;
    for (; j + 3 < cnt; j += 4) {
        a0 = ml_add(a0, ml_mul(a[j * stride], y[j]));
        a1 = ml_add(a1, ml_mul(a[(j + 1) * stride], y[j + 1]));
        a2 = ml_add(a2, ml_mul(a[(j + 2) * stride], y[j + 2]));
        a3 = ml_add(a3, ml_mul(a[(j + 3) * stride], y[j + 3]));
    }
    for (; j < cnt; ++j) a0 = ml_add(a0, ml_mul(a[j * stride], y[j]));
    return ml_add(ml_add(a0, a1), ml_add(a2, a3));
}

// x := L^{-T} L^{-1} x in one CTA (512 threads at 256 bits, 256 at 512 bits), blocked by NB with the inverted
// diagonal blocks: each block solve is a small matrix-vector product (one warp per
// output, a lane per term, tree-summed), then every thread updates one remaining row.
template <int N>
__global__ void __launch_bounds__(N <= 8 ? 512 : 256) potrs_blocked_kernel(int n, const mlf<N> *L, int ldl, const mlf<N> *Dinv, mlf<N> *x) {
    __shared__ mlf<N> ys[NB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int nblk = (n + NB - 1) / NB;
    // forward: L y = x
    for (int b = 0; b < nblk; ++b) {
        const int k0 = b * NB, kb = min(NB, n - k0);
        const mlf<N> *D = Dinv + (long long)b * NB * NB;
        for (int w = warp; w < kb; w += nwarps) {
            mlf<N> p = (lane <= w && lane < kb) ? ml_mul(D[w + NB * lane], x[k0 + lane]) : ml_zero<N>();
            p = ml_warp_sum(p);
            if (lane == 0) ys[w] = p;
        }
        __syncthreads();
        if (tid < kb) x[k0 + tid] = ys[tid];
        for (int i = k0 + kb + tid; i < n; i += blockDim.x) {
            const mlf<N> *Li = L + i + (long long)k0 * ldl;
            x[i] = ml_sub(x[i], dot_ld<N>(Li, ldl, ys, kb));
        }
        __syncthreads();
    }
    // backward: L^T z = y
    for (int b = nblk - 1; b >= 0; --b) {
        const int k0 = b * NB, kb = min(NB, n - k0);
        const mlf<N> *D = Dinv + (long long)b * NB * NB;
        for (int w = warp; w < kb; w += nwarps) {
            mlf<N> p = (lane >= w && lane < kb) ? ml_mul(D[lane + NB * w], x[k0 + lane]) : ml_zero<N>();
            p = ml_warp_sum(p);
            if (lane == 0) ys[w] = p;
        }
        __syncthreads();
        if (tid < kb) x[k0 + tid] = ys[tid];
        for (int i = tid; i < k0; i += blockDim.x) {
            const mlf<N> *Li = L + k0 + (long long)i * ldl;
            x[i] = ml_sub(x[i], dot_ld<N>(Li, 1, ys, kb));
        }
        __syncthreads();
    }
}

template <int N>
GemmProblem<N> gemm_nn(int M, int Nn, int K, const mlf<N> &alpha, const mlf<N> *A, long long lda, char ta,
                       const mlf<N> *B, long long ldb, char tb, const mlf<N> &beta, mlf<N> *C, long long ldc) {
    GemmProblem<N> p{};
    p.M = M;
    p.Nn = Nn;
    p.K = K;
    p.batch = 1;
    p.A = operand_A<N>(ta, A, lda, 0);
    p.B = operand_B<N>(tb, B, ldb, 0);
    p.C = C;
    p.ldc = ldc;
    p.sc = 0;
    p.alpha = alpha;
    p.beta = beta;
    p.lower_only = 0;
    return p;
}

}  // namespace

template <int N>
void ml_potrf(int n, mlf<N> *A, int lda, int *info, Workspace &ws, cudaStream_t s) {
    SDPG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
    const size_t mark = ws.used;
    mlf<N> *rinv = (mlf<N> *)ws.carve(NB * sizeof(mlf<N>));
    const mlf<N> mone = ml_from_int<N>(-1), one = ml_one<N>();
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0);
        mlf<N> *Akk = A + k0 + (long long)k0 * lda;
        potf2_kernel<N><<<1, 512, 0, s>>>(Akk, lda, kb, k0, info, rinv);
        SDPG_CHECK_LAUNCH();
        const int rows = n - k0 - kb;
        if (rows <= 0) break;
        mlf<N> *A21 = A + (k0 + kb) + (long long)k0 * lda;
        panel_trsm_kernel<N><<<ceil_div((long long)rows * 32, 256), 256, 0, s>>>(Akk, A21, lda, kb, rows, info, rinv);
        SDPG_CHECK_LAUNCH();
        GemmProblem<N> p = gemm_nn<N>(rows, rows, kb, mone, A21, lda, 'N', A21, lda, 'T', one,
                                      A + (k0 + kb) + (long long)(k0 + kb) * lda, lda);
        p.lower_only = 1;
        const size_t m2 = ws.used;
        ml_gemm<N>(p, ws, s);
        ws.used = m2;
    }
    ws.used = mark;
}

namespace {

template <int N>
__global__ void pad_lower_kernel(int n, int P, const mlf<N> *L, int ldl, mlf<N> *Lp) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)P * P) return;
    const int i = (int)(q % P), j = (int)(q / P);
    mlf<N> v = ml_zero<N>();
    if (i < n && j < n) {
        if (i >= j) v = L[i + (long long)j * ldl];
    } else if (i == j) {
        v = ml_one<N>();
    }
    Lp[q] = v;
}

template <int N>
__global__ void unpad_kernel(int n, int P, const mlf<N> *Xp, mlf<N> *X) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)n * n) return;
    const int i = (int)(q % n), j = (int)(q / n);
    X[q] = Xp[i + (long long)j * P];
}

inline int trtri_pad(int n) {
    int P = NB;
    while (P < n) P *= 2;
    return P;
}

}  // namespace

template <int N>
size_t ml_trtri_workspace_bytes(int n) {
    const int P = trtri_pad(n);
    const size_t pp = (size_t)P * P;
    GemmProblem<N> g{};
    g.M = P / 2;
    g.Nn = P / 2;
    g.K = P / 2;
    g.batch = 1;
    // padded L and X, the per-level W, and the scratch of the top level's GEMM (a level with
    // node size b quantises P*b/4 entries per operand, so the top level is the largest),
    // with slack for alignment
    return 2 * pp * sizeof(mlf<N>) + pp / 2 * sizeof(mlf<N>) + 2 * gemm_workspace_bytes<N>(g) + (64u << 10);
}

// Linv = L^{-1}: pad L to P = 32 * 2^k with an identity tail, invert the 32 x 32 diagonal
// blocks in parallel, then for node sizes b = 64, 128, ..., P form every node's
// off-diagonal block X21 = -X22 (L21 X11) with one batched GEMM pair per level.
template <int N>
void ml_trtri_lower(int n, const mlf<N> *L, int ldl, mlf<N> *Linv, Workspace &ws, cudaStream_t s) {
    const int P = trtri_pad(n);
    const size_t mark = ws.used;
    const long long pp = (long long)P * P;
    mlf<N> *Lp = (mlf<N> *)ws.carve(pp * sizeof(mlf<N>));
    mlf<N> *Xp = (mlf<N> *)ws.carve(pp * sizeof(mlf<N>));
    mlf<N> *W = (mlf<N> *)ws.carve(pp / 2 * sizeof(mlf<N>));
    pad_lower_kernel<N><<<ceil_div(pp, 256), 256, 0, s>>>(n, P, L, ldl, Lp);
    SDPG_CHECK_LAUNCH();
    SDPG_CUDA(cudaMemsetAsync(Xp, 0, pp * sizeof(mlf<N>), s));
    trtri_diag_kernel<N><<<P / NB, 256, 0, s>>>(Lp, P, Xp, P, P);
    SDPG_CHECK_LAUNCH();
    const mlf<N> one = ml_one<N>(), zero = ml_zero<N>(), mone = ml_from_int<N>(-1);
    for (int b = 2 * NB; b <= P; b *= 2) {
        const int h = b / 2, nodes = P / b;
        const long long node_stride = (long long)b * (1 + P);
        // W_t = L21 X11  (h x h x h), batched over nodes
        GemmProblem<N> p{};
        p.M = h;
        p.Nn = h;
        p.K = h;
        p.batch = nodes;
        p.A = operand_A<N>('N', Lp + h, P, node_stride);
        p.B = operand_B<N>('N', Xp, P, node_stride);
        p.C = W;
        p.ldc = h;
        p.sc = (long long)h * h;
        p.alpha = one;
        p.beta = zero;
        p.lower_only = 0;
        {
            const size_t m2 = ws.used;
            ml_gemm<N>(p, ws, s);
            ws.used = m2;
        }
        // X21 = -X22 W_t
        p.A = operand_A<N>('N', Xp + h + (long long)h * P, P, node_stride);
        p.B = operand_B<N>('N', W, h, (long long)h * h);
        p.C = Xp + h;
        p.ldc = P;
        p.sc = node_stride;
        p.alpha = mone;
        {
            const size_t m2 = ws.used;
            ml_gemm<N>(p, ws, s);
            ws.used = m2;
        }
    }
    unpad_kernel<N><<<ceil_div((long long)n * n, 256), 256, 0, s>>>(n, P, Xp, Linv);
    SDPG_CHECK_LAUNCH();
    ws.used = mark;
}

template <int N>
size_t ml_potrs_prepare_bytes(int n) {
    return (size_t)ceil_div(n, NB) * NB * NB * sizeof(mlf<N>);
}

template <int N>
void ml_potrs_prepare(int n, const mlf<N> *L, int ldl, mlf<N> *Dinv, cudaStream_t s) {
    trtri_diag_packed_kernel<N><<<ceil_div(n, NB), 256, 0, s>>>(L, ldl, Dinv, n);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void ml_potrs_solve(int n, const mlf<N> *L, int ldl, const mlf<N> *Dinv, mlf<N> *x, cudaStream_t s) {
    potrs_blocked_kernel<N><<<1, N <= 8 ? 512 : 256, 0, s>>>(n, L, ldl, Dinv, x);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void ml_potrs(int n, const mlf<N> *L, int ldl, mlf<N> *x, Workspace &ws, cudaStream_t s) {
    const size_t mark = ws.used;
    mlf<N> *Dinv = (mlf<N> *)ws.carve(ml_potrs_prepare_bytes<N>(n));
    ml_potrs_prepare<N>(n, L, ldl, Dinv, s);
    ml_potrs_solve<N>(n, L, ldl, Dinv, x, s);
    ws.used = mark;
}

#define SDPG_INST_CHOL(N)                                                                       \
    template void ml_potrf<N>(int, mlf<N> *, int, int *, Workspace &, cudaStream_t);            \
    template void ml_trtri_lower<N>(int, const mlf<N> *, int, mlf<N> *, Workspace &, cudaStream_t); \
    template size_t ml_trtri_workspace_bytes<N>(int);                                                       \
    template void ml_potrs<N>(int, const mlf<N> *, int, mlf<N> *, Workspace &, cudaStream_t);             \
    template size_t ml_potrs_prepare_bytes<N>(int);                                                        \
    template void ml_potrs_prepare<N>(int, const mlf<N> *, int, mlf<N> *, cudaStream_t);                    \
    template void ml_potrs_solve<N>(int, const mlf<N> *, int, const mlf<N> *, mlf<N> *, cudaStream_t);
SDPG_INST_CHOL(8)
SDPG_INST_CHOL(16)

}  // namespace sdpg
