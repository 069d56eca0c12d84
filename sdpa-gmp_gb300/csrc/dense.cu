// Elementwise, reduction, constraint and Schur-assembly kernels.
#include <string.h>

#include "kernels.cuh"
#include "mlwarp.cuh"

namespace sdpg {

namespace {

constexpr int kThreads = 256;

template <int N>
__host__ __device__ __forceinline__ bool is_one(const mlf<N> &a) {
    if (a.s || a.e != 1 || a.m[N - 1] != 0x80000000u) return false;
    for (int k = 0; k < N - 1; ++k)
        if (a.m[k]) return false;
    return true;
}

template <int N>
__global__ void axpby_kernel(long long n, mlf<N> a, const mlf<N> *x, mlf<N> b, const mlf<N> *y, mlf<N> *out,
                             int a_one, int b_mode) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    mlf<N> t = a_one ? x[i] : ml_mul(a, x[i]);
    if (b_mode == 1) t = ml_add(t, y[i]);
    else if (b_mode == 2) t = ml_add(t, ml_mul(b, y[i]));
    out[i] = t;
}

template <int N>
__global__ void copy_kernel(long long n, const mlf<N> *x, mlf<N> *out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = x[i];
}

template <int N>
__global__ void fill_kernel(long long n, mlf<N> *x, mlf<N> v) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}

template <int N>
__global__ void identity_kernel(int n, mlf<N> *A, mlf<N> v) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)n * n) return;
    const int r = (int)(i % n), c = (int)(i / n);
    A[i] = (r == c) ? v : ml_zero<N>();
}

// (A[i,j] + A[j,i]) / 2 into both, i < j (halving is exact: exponent - 1)
template <int N>
__global__ void symmetrize_kernel(int n, mlf<N> *A) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n || i >= j) return;
    mlf<N> *a = A + i + (long long)j * n;
    mlf<N> *b = A + j + (long long)i * n;
    const mlf<N> v = ml_ldexp(ml_add(*a, *b), -1);
    *a = v;
    *b = v;
}

template <int N>
__global__ void transpose_kernel(int n, const mlf<N> *A, mlf<N> *At) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n) return;
    At[j + (long long)i * n] = A[i + (long long)j * n];
}

template <int N>
__global__ void zero_upper_kernel(int n, mlf<N> *A) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n || i >= j) return;
    A[i + (long long)j * n] = ml_zero<N>();
}

// partial[b*G + blk] = sum over this block's strided share of x_b . y_b
template <int N>
__global__ void dot_partial_kernel(long long n, const mlf<N> *x, const long long *xoff, const mlf<N> *y,
                                   const long long *yoff, mlf<N> *partial) {
    const int b = blockIdx.y;
    const long long xo = xoff ? xoff[b] : 0, yo = yoff ? yoff[b] : 0;
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        a0 = ml_add(a0, ml_mul(x[xo + i], y[yo + i]));
        a1 = ml_add(a1, ml_mul(x[xo + i + stride], y[yo + i + stride]));
    }
    if (i < n) a0 = ml_add(a0, ml_mul(x[xo + i], y[yo + i]));
    mlf<N> acc = ml_block_sum(ml_add(a0, a1));
    if (threadIdx.x == 0) partial[(long long)b * gridDim.x + blockIdx.x] = acc;
}

template <int N>
__global__ void sum_partials_kernel(int G, const mlf<N> *partial, mlf<N> *out) {
    const int b = blockIdx.x;
    mlf<N> acc = ml_zero<N>();
    for (int i = threadIdx.x; i < G; i += blockDim.x) acc = ml_add(acc, partial[(long long)b * G + i]);
    acc = ml_block_sum(acc);
    if (threadIdx.x == 0) out[b] = acc;
}

template <int N>
__global__ void maxabs_partial_kernel(long long n, const mlf<N> *x, mlf<N> *partial) {
    mlf<N> acc = ml_zero<N>();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (ml_cmp_abs(x[i], acc) > 0) acc = x[i];
    acc = ml_block_maxabs(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = ml_abs(acc);
}

template <int N>
__global__ void maxabs_final_kernel(int G, const mlf<N> *partial, mlf<N> *out) {
    mlf<N> acc = ml_zero<N>();
    for (int i = threadIdx.x; i < G; i += blockDim.x)
        if (ml_cmp_abs(partial[i], acc) > 0) acc = partial[i];
    acc = ml_block_maxabs(acc);
    if (threadIdx.x == 0) out[0] = ml_abs(acc);
}

template <int N>
__global__ void trace_kernel(int n, const mlf<N> *A, mlf<N> *out) {
    mlf<N> acc = ml_zero<N>();
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc = ml_add(acc, A[i + (long long)i * n]);
    acc = ml_block_sum(acc);
    if (threadIdx.x == 0) out[0] = acc;
}

// ---- constraints ----

// one warp per sparse constraint: g[cid] += sum v * M[r, c]
template <int N>
__global__ void constraint_inner_sparse_kernel(BlockDev<N> B, const mlf<N> *M, mlf<N> *g) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= B.nc) return;
    if (B.dn_slot[warp] >= 0) return;
    mlf<N> acc = ml_zero<N>();
    for (int t = B.sp_off[warp] + lane; t < B.sp_off[warp + 1]; t += 32)
        acc = ml_add(acc, ml_mul(B.sp_val[t], M[B.sp_row[t] + (long long)B.sp_col[t] * B.n]));
    acc = ml_warp_sum(acc);
    if (lane == 0) {
        const int i = B.cid[warp];
        g[i] = ml_add(g[i], acc);
    }
}

template <int N>
__global__ void add_slots_kernel(int cnt, const int *cid, const mlf<N> *val, mlf<N> *g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const int i = cid[t];
    g[i] = ml_add(g[i], val[t]);
}

// M[e] = sum_d y[dn_cid[d]] * dense[d][e]  (dense constraints), or 0 when there are none
template <int N>
__global__ void constraint_plus_dense_kernel(BlockDev<N> B, const mlf<N> *y, mlf<N> *M) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nn = (long long)B.n * B.n;
    if (e >= nn) return;
    mlf<N> acc = ml_zero<N>();
    for (int d = 0; d < B.ndense; ++d) acc = ml_add(acc, ml_mul(y[B.dn_cid[d]], B.dense[(long long)d * nn + e]));
    M[e] = acc;
}

template <int N>
__global__ void constraint_plus_sparse_kernel(BlockDev<N> B, const mlf<N> *y, mlf<N> *M) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B.npos) return;
    mlf<N> acc = ml_zero<N>();
    for (int t = B.pos_off[p]; t < B.pos_off[p + 1]; ++t) acc = ml_add(acc, ml_mul(y[B.pos_k[t]], B.pos_v[t]));
    const int rc = B.pos_rc[p];
    M[rc] = ml_add(M[rc], acc);
}

// ---- Schur ----

template <int N>
__device__ __forceinline__ void schur_add(mlf<N> *bMat, int m, int i, int j, const mlf<N> &v) {
    if (i != j) {
        bMat[i + (long long)m * j] = ml_add(bMat[i + (long long)m * j], v);
        bMat[j + (long long)m * i] = ml_add(bMat[j + (long long)m * i], v);
    } else {
        bMat[i + (long long)m * i] = ml_add(bMat[i + (long long)m * i], v);
    }
}

template <int N>
__global__ void schur_f3_kernel(BlockDev<N> B, const mlf<N> *X, const mlf<N> *Zinv, mlf<N> *bMat, int m) {
    const int a = blockIdx.y * blockDim.y + threadIdx.y;  // owner (local)
    const int b = blockIdx.x * blockDim.x + threadIdx.x;  // partner (local)
    if (a >= B.nc || b >= B.nc) return;
    if (B.formula[a] != 2) return;
    if (B.rank[b] > B.rank[a]) return;
    const int n = B.n;
    mlf<N> acc = ml_zero<N>();
    for (int t1 = B.sp_off[b]; t1 < B.sp_off[b + 1]; ++t1) {
        const int al = B.sp_row[t1], be = B.sp_col[t1];
        mlf<N> sum = ml_zero<N>();
        for (int t2 = B.sp_off[a]; t2 < B.sp_off[a + 1]; ++t2) {
            const int ga = B.sp_row[t2], de = B.sp_col[t2];
            const mlf<N> pr = ml_mul(ml_mul(B.sp_val[t2], Zinv[de + (long long)n * be]), X[al + (long long)n * ga]);
            sum = ml_add(sum, pr);
        }
        acc = ml_add(acc, ml_mul(B.sp_val[t1], sum));
    }
    schur_add(bMat, m, B.cid[a], B.cid[b], acc);
}

template <int N>
__global__ void densify_kernel(BlockDev<N> B, const int *owners, int cnt, mlf<N> *out) {
    const long long nn = (long long)B.n * B.n;
    const int t = blockIdx.y;
    if (t >= cnt) return;
    const int a = owners[t];
    const int slot = B.dn_slot[a];
    mlf<N> *o = out + t * nn;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
        o[e] = (slot >= 0) ? B.dense[slot * nn + e] : ml_zero<N>();
}

template <int N>
__global__ void densify_scatter_kernel(BlockDev<N> B, const int *owners, int cnt, mlf<N> *out) {
    const long long nn = (long long)B.n * B.n;
    const int t = blockIdx.y;
    if (t >= cnt) return;
    const int a = owners[t];
    if (B.dn_slot[a] >= 0) return;
    mlf<N> *o = out + t * nn;
    for (int q = B.sp_off[a] + blockIdx.x * blockDim.x + threadIdx.x; q < B.sp_off[a + 1]; q += gridDim.x * blockDim.x)
        o[B.sp_row[q] + (long long)B.n * B.sp_col[q]] = B.sp_val[q];  // entries are unique
}

template <int N>
__global__ void schur_f1_sparse_kernel(BlockDev<N> B, const int *owners, int cnt, const mlf<N> *G, mlf<N> *bMat,
                                       int m) {
    const int t = blockIdx.y * blockDim.y + threadIdx.y;  // owner slot
    const int b = blockIdx.x * blockDim.x + threadIdx.x;  // partner local index
    if (t >= cnt || b >= B.nc) return;
    const int a = owners[t];
    if (B.dn_slot[b] >= 0) return;  // dense partners handled separately
    if (B.rank[b] > B.rank[a]) return;
    const long long nn = (long long)B.n * B.n;
    const mlf<N> *Gt = G + t * nn;
    mlf<N> acc = ml_zero<N>();
    for (int q = B.sp_off[b]; q < B.sp_off[b + 1]; ++q)
        acc = ml_add(acc, ml_mul(B.sp_val[q], Gt[B.sp_row[q] + (long long)B.n * B.sp_col[q]]));
    schur_add(bMat, m, B.cid[a], B.cid[b], acc);
}

// P[t + cnt*d]: owner slot t times dense slot d
template <int N>
__global__ void schur_f1_dense_scatter_kernel(BlockDev<N> B, const int *owners, int cnt, const mlf<N> *P,
                                              mlf<N> *bMat, int m, const int *dense_local) {
    const int t = blockIdx.y * blockDim.y + threadIdx.y;
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt || d >= B.ndense) return;
    const int a = owners[t];
    const int b = dense_local[d];
    if (B.rank[b] > B.rank[a]) return;
    schur_add(bMat, m, B.cid[a], B.cid[b], P[t + (long long)cnt * d]);
}

inline int grid1(long long n, int t = kThreads) { return (int)((n + t - 1) / t); }

}  // namespace

template <int N>
void k_axpby(long long n, const mlf<N> &a, const mlf<N> *x, const mlf<N> &b, const mlf<N> *y, mlf<N> *out,
             cudaStream_t s) {
    if (n <= 0) return;
    const int b_mode = (ml_is_zero(b) || y == nullptr) ? 0 : (is_one(b) ? 1 : 2);
    SDPG_KT_BEGIN(s);
    axpby_kernel<N><<<grid1(n), kThreads, 0, s>>>(n, a, x, b, y, out, is_one(a) ? 1 : 0, b_mode);
    SDPG_CHECK_LAUNCH_KT("axpby_kernel", s);
}

template <int N>
void k_copy(long long n, const mlf<N> *x, mlf<N> *out, cudaStream_t s) {
    if (n <= 0) return;
    SDPG_CUDA(cudaMemcpyAsync(out, x, n * sizeof(mlf<N>), cudaMemcpyDeviceToDevice, s));
}

template <int N>
void k_fill(long long n, mlf<N> *x, const mlf<N> &v, cudaStream_t s) {
    if (n <= 0) return;
    SDPG_KT_BEGIN(s);
    fill_kernel<N><<<grid1(n), kThreads, 0, s>>>(n, x, v);
    SDPG_CHECK_LAUNCH_KT("fill_kernel", s);
}

template <int N>
void k_set_identity(int n, mlf<N> *A, const mlf<N> &v, cudaStream_t s) {
    SDPG_KT_BEGIN(s);
    identity_kernel<N><<<grid1((long long)n * n), kThreads, 0, s>>>(n, A, v);
    SDPG_CHECK_LAUNCH_KT("identity_kernel", s);
}

template <int N>
void k_symmetrize(int n, mlf<N> *A, cudaStream_t s) {
    dim3 blk(16, 16), g(ceil_div(n, 16), ceil_div(n, 16));
    SDPG_KT_BEGIN(s);
    symmetrize_kernel<N><<<g, blk, 0, s>>>(n, A);
    SDPG_CHECK_LAUNCH_KT("symmetrize_kernel", s);
}

template <int N>
void k_transpose(int n, const mlf<N> *A, mlf<N> *At, cudaStream_t s) {
    dim3 blk(16, 16), g(ceil_div(n, 16), ceil_div(n, 16));
    SDPG_KT_BEGIN(s);
    transpose_kernel<N><<<g, blk, 0, s>>>(n, A, At);
    SDPG_CHECK_LAUNCH_KT("transpose_kernel", s);
}

template <int N>
void k_zero_strict_upper(int n, mlf<N> *A, cudaStream_t s) {
    dim3 blk(16, 16), g(ceil_div(n, 16), ceil_div(n, 16));
    SDPG_KT_BEGIN(s);
    zero_upper_kernel<N><<<g, blk, 0, s>>>(n, A);
    SDPG_CHECK_LAUNCH_KT("zero_upper_kernel", s);
}

template <int N>
void k_dot_batched(long long n, const mlf<N> *x, const long long *xoff, const mlf<N> *y, const long long *yoff,
                   int batch, mlf<N> *out, Workspace &ws, cudaStream_t s) {
    if (batch <= 0) return;
    // a single dot: about two products per thread (short multiply-add chains: these dots
    // are latency-bound), at most 1024 partial sums; batched dots keep eight products per
    // thread and at most 64 partials each (the workspace their callers reserve)
    const int per = batch == 1 ? 2 : 8, gmax = batch == 1 ? 1024 : 64;
    int G = (int)((n + kThreads * per - 1) / (kThreads * per));
    if (G < 1) G = 1;
    if (G > gmax) G = gmax;
    mlf<N> *partial = (mlf<N> *)ws.carve((size_t)G * batch * sizeof(mlf<N>));
    dim3 g(G, batch);
    SDPG_KT_BEGIN(s);
    dot_partial_kernel<N><<<g, kThreads, 0, s>>>(n, x, xoff, y, yoff, partial);
    SDPG_CHECK_LAUNCH_KT("dot_partial_kernel", s);
    SDPG_KT_BEGIN(s);
    sum_partials_kernel<N><<<batch, kThreads, 0, s>>>(G, partial, out);
    SDPG_CHECK_LAUNCH_KT("sum_partials_kernel", s);
}

template <int N>
void k_dot(long long n, const mlf<N> *x, const mlf<N> *y, mlf<N> *out, Workspace &ws, cudaStream_t s) {
    k_dot_batched<N>(n, x, nullptr, y, nullptr, 1, out, ws, s);
}

template <int N>
void k_maxabs(long long n, const mlf<N> *x, mlf<N> *out, Workspace &ws, cudaStream_t s) {
    int G = (int)((n + kThreads * 8 - 1) / (kThreads * 8));
    if (G < 1) G = 1;
    if (G > 64) G = 64;
    mlf<N> *partial = (mlf<N> *)ws.carve((size_t)G * sizeof(mlf<N>));
    SDPG_KT_BEGIN(s);
    maxabs_partial_kernel<N><<<G, kThreads, 0, s>>>(n, x, partial);
    SDPG_CHECK_LAUNCH_KT("maxabs_partial_kernel", s);
    SDPG_KT_BEGIN(s);
    maxabs_final_kernel<N><<<1, 64, 0, s>>>(G, partial, out);
    SDPG_CHECK_LAUNCH_KT("maxabs_final_kernel", s);
}

template <int N>
void k_trace(int n, const mlf<N> *A, mlf<N> *out, cudaStream_t s) {
    SDPG_KT_BEGIN(s);
    trace_kernel<N><<<1, kThreads, 0, s>>>(n, A, out);
    SDPG_CHECK_LAUNCH_KT("trace_kernel", s);
}

template <int N>
void k_constraint_inner(const BlockDev<N> &B, const mlf<N> *M, mlf<N> *g, Workspace &ws, cudaStream_t s) {
    if (B.nc == 0) return;
    SDPG_KT_BEGIN(s);
    constraint_inner_sparse_kernel<N><<<grid1((long long)B.nc * 32), kThreads, 0, s>>>(B, M, g);
    SDPG_CHECK_LAUNCH_KT("constraint_inner_sparse_kernel", s);
    if (B.ndense > 0) {
        const long long nn = (long long)B.n * B.n;
        mlf<N> *tmp = (mlf<N> *)ws.carve((size_t)B.ndense * sizeof(mlf<N>));
        k_dot_batched<N>(nn, B.dense, B.dn_off, M, nullptr, B.ndense, tmp, ws, s);
        SDPG_KT_BEGIN(s);
        add_slots_kernel<N><<<grid1(B.ndense), kThreads, 0, s>>>(B.ndense, B.dn_cid, tmp, g);
        SDPG_CHECK_LAUNCH_KT("add_slots_kernel", s);
    }
}

template <int N>
void k_constraint_plus(const BlockDev<N> &B, const mlf<N> *y, mlf<N> *M, cudaStream_t s) {
    const long long nn = (long long)B.n * B.n;
    SDPG_KT_BEGIN(s);
    constraint_plus_dense_kernel<N><<<grid1(nn), kThreads, 0, s>>>(B, y, M);
    SDPG_CHECK_LAUNCH_KT("constraint_plus_dense_kernel", s);
    if (B.npos > 0) {
        SDPG_KT_BEGIN(s);
        constraint_plus_sparse_kernel<N><<<grid1(B.npos), kThreads, 0, s>>>(B, y, M);
        SDPG_CHECK_LAUNCH_KT("constraint_plus_sparse_kernel", s);
    }
}

template <int N>
void k_schur_f3(const BlockDev<N> &B, const mlf<N> *X, const mlf<N> *Zinv, mlf<N> *bMat, int m, cudaStream_t s) {
    if (B.nc == 0) return;
    dim3 blk(32, 8), g(ceil_div(B.nc, 32), ceil_div(B.nc, 8));
    SDPG_KT_BEGIN(s);
    schur_f3_kernel<N><<<g, blk, 0, s>>>(B, X, Zinv, bMat, m);
    SDPG_CHECK_LAUNCH_KT("schur_f3_kernel", s);
}

template <int N>
void k_densify(const BlockDev<N> &B, const int *owners, int cnt, mlf<N> *out, cudaStream_t s) {
    if (cnt <= 0) return;
    const long long nn = (long long)B.n * B.n;
    int gx = grid1(nn);
    if (gx > 256) gx = 256;
    SDPG_KT_BEGIN(s);
    densify_kernel<N><<<dim3(gx, cnt), kThreads, 0, s>>>(B, owners, cnt, out);
    SDPG_CHECK_LAUNCH_KT("densify_kernel", s);
    SDPG_KT_BEGIN(s);
    densify_scatter_kernel<N><<<dim3(gx, cnt), kThreads, 0, s>>>(B, owners, cnt, out);
    SDPG_CHECK_LAUNCH_KT("densify_scatter_kernel", s);
}

template <int N>
void k_schur_f1_sparse(const BlockDev<N> &B, const int *owners, int cnt, const mlf<N> *G, mlf<N> *bMat, int m,
                       cudaStream_t s) {
    if (cnt <= 0 || B.nc == 0) return;
    dim3 blk(32, 8), g(ceil_div(B.nc, 32), ceil_div(cnt, 8));
    SDPG_KT_BEGIN(s);
    schur_f1_sparse_kernel<N><<<g, blk, 0, s>>>(B, owners, cnt, G, bMat, m);
    SDPG_CHECK_LAUNCH_KT("schur_f1_sparse_kernel", s);
}

template <int N>
void k_schur_f1_dense_scatter(const BlockDev<N> &B, const int *owners, int cnt, const mlf<N> *P, mlf<N> *bMat,
                              int m, cudaStream_t s) {
    if (cnt <= 0 || B.ndense == 0) return;
    dim3 blk(32, 8), g(ceil_div(B.ndense, 32), ceil_div(cnt, 8));
    SDPG_KT_BEGIN(s);
    schur_f1_dense_scatter_kernel<N><<<g, blk, 0, s>>>(B, owners, cnt, P, bMat, m, B.dn_local);
    SDPG_CHECK_LAUNCH_KT("schur_f1_dense_scatter_kernel", s);
}

#define SDPG_INST_DENSE(N)                                                                                   \
    template void k_axpby<N>(long long, const mlf<N> &, const mlf<N> *, const mlf<N> &, const mlf<N> *,        \
                             mlf<N> *, cudaStream_t);                                                        \
    template void k_copy<N>(long long, const mlf<N> *, mlf<N> *, cudaStream_t);                              \
    template void k_fill<N>(long long, mlf<N> *, const mlf<N> &, cudaStream_t);                              \
    template void k_set_identity<N>(int, mlf<N> *, const mlf<N> &, cudaStream_t);                            \
    template void k_symmetrize<N>(int, mlf<N> *, cudaStream_t);                                              \
    template void k_transpose<N>(int, const mlf<N> *, mlf<N> *, cudaStream_t);                               \
    template void k_zero_strict_upper<N>(int, mlf<N> *, cudaStream_t);                                       \
    template void k_dot_batched<N>(long long, const mlf<N> *, const long long *, const mlf<N> *,             \
                                   const long long *, int, mlf<N> *, Workspace &, cudaStream_t);             \
    template void k_dot<N>(long long, const mlf<N> *, const mlf<N> *, mlf<N> *, Workspace &, cudaStream_t);  \
    template void k_maxabs<N>(long long, const mlf<N> *, mlf<N> *, Workspace &, cudaStream_t);               \
    template void k_trace<N>(int, const mlf<N> *, mlf<N> *, cudaStream_t);                                   \
    template void k_constraint_inner<N>(const BlockDev<N> &, const mlf<N> *, mlf<N> *, Workspace &,          \
                                        cudaStream_t);                                                       \
    template void k_constraint_plus<N>(const BlockDev<N> &, const mlf<N> *, mlf<N> *, cudaStream_t);         \
    template void k_schur_f3<N>(const BlockDev<N> &, const mlf<N> *, const mlf<N> *, mlf<N> *, int,          \
                                cudaStream_t);                                                               \
    template void k_densify<N>(const BlockDev<N> &, const int *, int, mlf<N> *, cudaStream_t);               \
    template void k_schur_f1_sparse<N>(const BlockDev<N> &, const int *, int, const mlf<N> *, mlf<N> *, int, \
                                       cudaStream_t);                                                        \
    template void k_schur_f1_dense_scatter<N>(const BlockDev<N> &, const int *, int, const mlf<N> *,         \
                                              mlf<N> *, int, cudaStream_t);
SDPG_INST_DENSE(8)
SDPG_INST_DENSE(16)

}  // namespace sdpg
