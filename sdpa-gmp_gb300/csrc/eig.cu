// Minimum-eigenvalue machinery for the step length
// (StepLength::computeStepLength -> Jal::getMinEigen, sdpa_parts.cpp:298-360,
// sdpa_jordan.cpp:55-88):
//   * matrix-vector products for the Lanczos recurrence (Lal::getMinEigen,
//     sdpa_linear.cpp:27-124: Rtrmv^T, Rgemv, Rtrmv);
//   * the smallest eigenvalue of a symmetric tridiagonal matrix and the last
//     component of its unit eigenvector (what the reference reads from
//     Rsteqr's output: out.ele[0] and Q.de_ele[k]);
//   * Householder tridiagonalisation for blocks of size <= 20 (the Rsyev path,
//     sdpa_linear.cpp:126-158: Rsytrd + Rsterf).
//
// Tridiagonal method: bisection with Sturm counts in double precision brackets
// the smallest eigenvalue; Newton's method on the monic characteristic
// polynomial p_k (three-term recurrence, run in multi-limb arithmetic) then
// converges quadratically to full precision.  With p_{k-1} the polynomial of the
// leading (k-1) x (k-1) block, the squared last eigenvector component is
// p_{k-1}(lambda) / p_k'(lambda).
#include <float.h>

#include <algorithm>
#include <climits>
#include <mutex>

#include "kernels.cuh"
#include "mlwarp.cuh"

namespace sdpg {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxTri = 512;

// y[o] = sum_i A[i,o] x[i]  (op 'T': columns of A), tri: 0 all rows, 1 rows i >= o, 2 rows i <= o
template <int N>
__global__ void matvec_t_kernel(int n, const mlf<N> *A, int tri, const mlf<N> *x, mlf<N> *y,
                                const int *gate = nullptr) {
    const int o = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (o >= n || (gate && !*gate)) return;
    const int lo = (tri == 1) ? o : 0;
    const int hi = (tri == 2) ? o + 1 : n;
    const mlf<N> *col = A + (long long)o * n;
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
    int i = lo + lane;
    for (; i + 32 < hi; i += 64) {
        a0 = ml_add(a0, ml_mul(col[i], x[i]));
        a1 = ml_add(a1, ml_mul(col[i + 32], x[i + 32]));
    }
    if (i < hi) a0 = ml_add(a0, ml_mul(col[i], x[i]));
    mlf<N> acc = ml_warp_sum(ml_add(a0, a1));
    if (lane == 0) y[o] = acc;
}

// The same with four warps per output (each a quarter of the rows, combined in shared
// memory): four times the warps in flight for the single-vector products of Lanczos.
constexpr int kMvSplit = 4;
template <int N>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    matvec_t_split_kernel(int n, const mlf<N> *A, int tri, const mlf<N> *x, mlf<N> *y, const int *gate) {
    constexpr int kOut = kWarpsPerBlock / kMvSplit;
    __shared__ mlf<N> part[kWarpsPerBlock];
    if (gate && !*gate) return;  // a device-controlled Lanczos run that has stopped
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int o = blockIdx.x * kOut + warp / kMvSplit, sp = warp % kMvSplit;
    mlf<N> acc = ml_zero<N>();
    if (o < n) {
        const int lo = (tri == 1) ? o : 0;
        const int hi = (tri == 2) ? o + 1 : n;
        const mlf<N> *col = A + (long long)o * n;
        mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
        int i = lo + sp * 32 + lane;
        for (; i + 32 * kMvSplit < hi; i += 64 * kMvSplit) {
            a0 = ml_add(a0, ml_mul(col[i], x[i]));
            a1 = ml_add(a1, ml_mul(col[i + 32 * kMvSplit], x[i + 32 * kMvSplit]));
        }
        if (i < hi) a0 = ml_add(a0, ml_mul(col[i], x[i]));
        acc = ml_warp_sum(ml_add(a0, a1));
    }
    if (lane == 0) part[warp] = acc;
    __syncthreads();
    const int oo = blockIdx.x * kOut + (int)threadIdx.x;
    if ((int)threadIdx.x < kOut && oo < n) {
        const mlf<N> *pp = part + threadIdx.x * kMvSplit;
        y[oo] = ml_add(ml_add(pp[0], pp[1]), ml_add(pp[2], pp[3]));
    }
}

// y[o] = sum_j A[o,j] x[j]  (op 'N': rows of A)
template <int N>
__global__ void matvec_n_kernel(int n, const mlf<N> *A, int tri, const mlf<N> *x, mlf<N> *y) {
    const int o = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (o >= n) return;
    const int lo = (tri == 2) ? o : 0;      // upper: columns j >= o
    const int hi = (tri == 1) ? o + 1 : n;  // lower: columns j <= o
    mlf<N> acc = ml_zero<N>();
    for (int j = lo + lane; j < hi; j += 32) acc = ml_add(acc, ml_mul(A[o + (long long)j * n], x[j]));
    acc = ml_warp_sum(acc);
    if (lane == 0) y[o] = acc;
}

// Number of eigenvalues of the (scaled, single-precision) tridiagonal below x: the
// negative pivots of the LDL^T factorisation of T - x I (Sturm sequence).
__device__ int sturm_count_f(int k, const float *d, const float *e2, float x) {
    int cnt = 0;
    float q = d[0] - x;
    cnt += q < 0.0f;
    for (int i = 1; i < k; ++i) {
        if (q == 0.0f) q = -1e-30f;
        q = (d[i] - x) - e2[i - 1] / q;
        cnt += q < 0.0f;
    }
    return cnt;
}

// a * 2^-E as a float (0 below the float range); E is at least a's exponent
template <int N>
__device__ float ml_to_float_scaled(const mlf<N> &a, int E) {
    if (ml_is_zero(a)) return 0.0f;
    const int ex = a.e - E;
    if (ex < -120) return 0.0f;
    const float f = ldexpf((float)(a.m[N - 1] >> 8) * 5.9604644775390625e-8f, ex);
    return a.s ? -f : f;
}

// an mlf value from another lane of the two lanes (0 and 1) that evaluate the recurrences
template <int M>
__device__ __forceinline__ mlf<M> ml_shfl2(const mlf<M> &v, int src) {
    mlf<M> r;
    r.e = __shfl_sync(0x3u, v.e, src);
    r.s = __shfl_sync(0x3u, v.s, src);
#pragma unroll
    for (int w = 0; w < M; ++w) r.m[w] = __shfl_sync(0x3u, v.m[w], src);
    return r;
}

// p_k(lam), p_k'(lam) and p_{k-1}(lam) of det(lam I - T) at M limbs, from the diagonal d
// and the squared off-diagonal b2 held at N limbs in shared memory.  Lanes 0 and 1 of the
// warp run it together: lane 0 the recurrence p_i = a_i p_{i-1} - b2 p_{i-2}, lane 1 its
// derivative p_i' = p_{i-1} + a_i p_{i-1}' - b2 p_{i-2}' (a_i = lam - d_i), which takes
// p_{i-1} from lane 0 each step; both lanes return all three values.
template <int M, int N>
__device__ void charpoly_at(int k, const mlf<N> *d, const mlf<N> *b2s, const mlf<M> &lam, mlf<M> *pk, mlf<M> *dpk,
                            mlf<M> *pkm1) {
    const bool deriv = (threadIdx.x & 1) != 0;
    const mlf<M> p1 = ml_sub(lam, ml_narrow<M, N>(d[0]));
    mlf<M> x_prev = deriv ? ml_zero<M>() : ml_one<M>();
    mlf<M> x_cur = deriv ? ml_one<M>() : p1;
    mlf<M> p_cur = p1;  // p_{i-1}, the derivative lane's extra term
    for (int i = 1; i < k; ++i) {
        const mlf<M> a = ml_sub(lam, ml_narrow<M, N>(d[i]));
        const mlf<M> b2 = ml_narrow<M, N>(b2s[i - 1]);
        mlf<M> x_new = ml_sub(ml_mul(a, x_cur), ml_mul(b2, x_prev));
        if (deriv) x_new = ml_add(x_new, p_cur);
        p_cur = ml_shfl2(x_new, 0);
        x_prev = x_cur;
        x_cur = x_new;
    }
    *pk = ml_shfl2(x_cur, 0);
    *pkm1 = ml_shfl2(x_prev, 0);
    *dpk = ml_shfl2(x_cur, 1);
}

// a / b to about H limbs of relative precision, returned at M limbs
template <int H, int M>
__device__ __forceinline__ mlf<M> ml_div_half(const mlf<M> &a, const mlf<M> &b) {
    if constexpr (H >= M) {
        return mlc_div(a, b);
    } else {
        return ml_widen<M, H>(mlc_div(ml_narrow<H, M>(a), ml_narrow<H, M>(b)));
    }
}

// Newton on det(lam I - T) at M limbs until the step is below 2^-tol of the scale
// 2^scale_e (at most maxit evaluations).  Returns 1 when that tolerance was met.  The
// step p_k / p_k' is formed at half precision: entering a step with relative error e,
// the step is about e, so a quotient good to half of M's bits leaves an error of order
// e 2^-(16 M), below the quadratic term's.  Run by lanes 0 and 1 together.
template <int M, int N>
__device__ int newton_level(int k, const mlf<N> *d, const mlf<N> *b2s, mlf<M> &lam, int scale_e, int tol, int maxit,
                            mlf<M> *pkm1, mlf<M> *dpk) {
    constexpr int H = M / 2 > 2 ? M / 2 : 2;
    int prev_e = INT_MAX;
    for (int it = 0; it < maxit; ++it) {
        mlf<M> pk;
        charpoly_at<M, N>(k, d, b2s, lam, &pk, dpk, pkm1);
        if (ml_is_zero(pk)) return 1;
        if (ml_is_zero(*dpk)) return 0;
        const mlf<M> delta = ml_div_half<H, M>(pk, *dpk);
        lam = mlc_sub(lam, delta);
        if (ml_is_zero(delta) || delta.e < scale_e - tol) return 1;
        // steps that no longer shrink fourfold: the rounding floor of the recurrence
        if (delta.e > prev_e - 2) return 1;
        // quadratic convergence: the error left after this step is about C delta^2 with
        // C ~ delta / delta_prev^2; stop when that is already below the tolerance
        if (prev_e != INT_MAX && 3 * delta.e - 2 * prev_e < scale_e - tol - 4) return 1;
        prev_e = delta.e;
    }
    return 0;
}

// Smallest eigenvalue of tridiag(e, d, e): a 32-way single-precision multisection of
// the Gershgorin interval on the Sturm count (one point per lane) down to about 20
// bits, then Newton's method on the characteristic polynomial from the left end of
// the bracket at 4, 8, ... limbs up to full precision (from the left of the smallest
// root of a real-rooted polynomial, Newton increases monotonically towards it), on
// lanes 0 and 1.  out[1] = |z_k| = sqrt(p_{k-1}(lam) / p_k'(lam)).
// Run by one whole warp; `tri` is shared memory for 2k values (the k diagonal entries,
// then the k - 1 squared off-diagonals).
template <int N>
__device__ void tridiag_min_warp(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status, mlf<N> *tri) {
    __shared__ float df[kMaxTri], e2f[kMaxTri];
    __shared__ float bounds[2];
    const int lane = threadIdx.x & 31;
    if (k <= 0 || k > kMaxTri) {
        if (lane == 0) *status = 1;
        return;
    }
    if (k == 1) {
        if (lane == 0) {
            out[0] = d[0];
            out[1] = ml_one<N>();
            *status = 0;
        }
        return;
    }
    // common scale 2^E: the largest exponent among the entries
    int E = INT_MIN;
    for (int i = lane; i < k; i += 32) {
        if (!ml_is_zero(d[i])) E = max(E, d[i].e);
        if (i + 1 < k && !ml_is_zero(e[i])) E = max(E, e[i].e);
    }
    for (int o = 16; o > 0; o >>= 1) E = max(E, __shfl_xor_sync(0xffffffffu, E, o));
    if (E == INT_MIN) {  // the zero matrix
        if (lane == 0) {
            out[0] = ml_zero<N>();
            out[1] = ml_one<N>();
            *status = 0;
        }
        return;
    }
    float lo = 3.4e38f, hi = -3.4e38f;
    for (int i = lane; i < k; i += 32) {
        const float di = ml_to_float_scaled(d[i], E);
        const float em = i > 0 ? fabsf(ml_to_float_scaled(e[i - 1], E)) : 0.0f;
        const float ep = i + 1 < k ? fabsf(ml_to_float_scaled(e[i], E)) : 0.0f;
        df[i] = di;
        if (i + 1 < k) e2f[i] = ep * ep;
        lo = fminf(lo, di - em - ep);
        hi = fmaxf(hi, di + em + ep);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __syncwarp();
    // widen slightly: the float Gershgorin bounds are rounded
    const float span = fmaxf(hi - lo, 1e-30f);
    lo -= 1e-6f * span + 1e-30f;
    hi += 1e-6f * span + 1e-30f;
    const float scale = fmaxf(fabsf(lo), fabsf(hi));  // matrix scale for the stopping rules
    for (int round = 0; round < 8; ++round) {
        const float w = hi - lo;
        if (w <= 1e-6f * fmaxf(fmaxf(fabsf(lo), fabsf(hi)), 1e-30f)) break;
        const float x = lo + w * (float)(lane + 1) * (1.0f / 33.0f);
        const unsigned ball = __ballot_sync(0xffffffffu, sturm_count_f(k, df, e2f, x) >= 1);
        const int first = ball ? __ffs(ball) - 1 : 32;  // first point with an eigenvalue below it
        const float xlo = __shfl_sync(0xffffffffu, x, first > 0 ? first - 1 : 0);
        const float xhi = __shfl_sync(0xffffffffu, x, first < 32 ? first : 31);
        if (first == 32) lo = xhi;
        else {
            hi = xhi;
            if (first > 0) lo = xlo;
        }
    }
    if (lane == 0) {
        bounds[0] = lo;
        bounds[1] = hi;
    }
    mlf<N> *ds = tri;
    mlf<N> *b2s = ds + k;
    for (int i = lane; i < k; i += 32) {
        ds[i] = d[i];
        if (i + 1 < k) b2s[i] = ml_mul(e[i], e[i]);
    }
    __syncwarp();
    if (lane >= 2) return;  // lanes 0 and 1 evaluate the recurrences (charpoly_at)
    const int scale_e = E + ilogbf(scale) + 1;
    mlf<N> lam, pkm1, dpk;
    int ok;
    if constexpr (N <= 4) {
        lam = ml_ldexp(ml_from_float<N>(bounds[0]), E);
        ok = newton_level<N, N>(k, ds, b2s, lam, scale_e, 32 * N - 4, 10, &pkm1, &dpk);
    } else {
        // from the ~20-bit float bracket straight to 4 limbs: a 2-limb step costs about
        // as much as a 4-limb one here, so three 4-limb steps (20 -> 40 -> 80 -> 124 bits)
        // replace two of each
        mlf<4> l4 = ml_ldexp(ml_from_float<4>(bounds[0]), E);
        {
            mlf<4> a, b;
            newton_level<4, N>(k, ds, b2s, l4, scale_e, 110, 8, &a, &b);
        }
        if constexpr (N <= 8) {
            lam = ml_widen<N, 4>(l4);
        } else {
            mlf<8> l8 = ml_widen<8, 4>(l4);
            mlf<8> a, b;
            newton_level<8, N>(k, ds, b2s, l8, scale_e, 230, 6, &a, &b);
            lam = ml_widen<N, 8>(l8);
        }
        ok = newton_level<N, N>(k, ds, b2s, lam, scale_e, 32 * N - 4, 8, &pkm1, &dpk);
    }
    // |z_k| = sqrt(p_{k-1} / p_k') = |p_{k-1}| / sqrt(|p_{k-1} p_k'|): one inverse square
    // root instead of a quotient and a square root
    const mlf<N> prod = ml_abs(mlc_mul(pkm1, dpk));
    const mlf<N> z = ml_is_zero(prod) ? ml_zero<N>() : mlc_mul(ml_abs(pkm1), mlc_rsqrt(prod));
    if (lane == 0) {
        out[0] = lam;
        out[1] = z;
        *status = ok ? 0 : 2;
    }
}

template <int N>
__global__ void tridiag_min_kernel(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status,
                                   const int *gate) {
    extern __shared__ uint8_t tri_smem[];
    if (gate && !*gate) return;  // a device-controlled Lanczos run that has stopped
    tridiag_min_warp<N>(k, d, e, out, status, reinterpret_cast<mlf<N> *>(tri_smem));
}

// Householder reduction of the symmetric n x n A (lower triangle used) to tridiagonal form.
template <int N>
__global__ void tridiagonalize_kernel(int n, mlf<N> *A, mlf<N> *dout, mlf<N> *eout) {
    __shared__ mlf<N> v[64], p[64], w[64];
    __shared__ mlf<N> tau_s, K_s, beta_s;
    __shared__ int skip;
    const int tid = threadIdx.x;
    // symmetrise from the lower triangle
    for (int q = tid; q < n * n; q += blockDim.x) {
        const int i = q % n, j = q / n;
        if (i < j) A[i + (long long)j * n] = A[j + (long long)i * n];
    }
    __syncthreads();
    for (int j = 0; j + 2 < n; ++j) {
        const int L = n - j - 1;  // length of x = A[j+1:n, j]
        if (tid == 0) {
            const mlf<N> x0 = A[(j + 1) + (long long)j * n];
            mlf<N> sigma = ml_zero<N>();
            for (int i = 1; i < L; ++i) {
                const mlf<N> xi = A[(j + 1 + i) + (long long)j * n];
                sigma = ml_add(sigma, ml_mul(xi, xi));
            }
            if (ml_is_zero(sigma)) {
                skip = 1;
                beta_s = x0;
            } else {
                skip = 0;
                const mlf<N> mu = ml_sqrt(ml_add(ml_mul(x0, x0), sigma));
                const mlf<N> beta = (x0.s == 0) ? ml_neg(mu) : mu;  // -sign(x0) * mu
                const mlf<N> v0 = ml_sub(x0, beta);
                tau_s = ml_div(ml_sub(beta, x0), beta);
                beta_s = beta;
                const mlf<N> rv0 = ml_recip(v0);
                v[0] = ml_one<N>();
                for (int i = 1; i < L; ++i) v[i] = ml_mul(A[(j + 1 + i) + (long long)j * n], rv0);
            }
        }
        __syncthreads();
        if (!skip) {
            // p = tau * A22 v
            for (int i = tid; i < L; i += blockDim.x) {
                mlf<N> acc = ml_zero<N>();
                for (int c = 0; c < L; ++c) acc = ml_add(acc, ml_mul(A[(j + 1 + i) + (long long)(j + 1 + c) * n], v[c]));
                p[i] = ml_mul(tau_s, acc);
            }
            __syncthreads();
            if (tid == 0) {
                mlf<N> acc = ml_zero<N>();
                for (int i = 0; i < L; ++i) acc = ml_add(acc, ml_mul(v[i], p[i]));
                K_s = ml_ldexp(ml_mul(tau_s, acc), -1);
            }
            __syncthreads();
            for (int i = tid; i < L; i += blockDim.x) w[i] = ml_sub(p[i], ml_mul(K_s, v[i]));
            __syncthreads();
            for (int q = tid; q < L * L; q += blockDim.x) {
                const int r = q % L, c = q / L;
                mlf<N> *a = A + (j + 1 + r) + (long long)(j + 1 + c) * n;
                *a = ml_sub(*a, ml_add(ml_mul(v[r], w[c]), ml_mul(w[r], v[c])));
            }
        }
        __syncthreads();
        if (tid == 0) {
            dout[j] = A[j + (long long)j * n];
            eout[j] = beta_s;
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            dout[n - 2] = A[(n - 2) + (long long)(n - 2) * n];
            eout[n - 2] = A[(n - 1) + (long long)(n - 2) * n];
        }
        dout[n - 1] = A[(n - 1) + (long long)(n - 1) * n];
    }
}

}  // namespace

template <int N>
void k_matvec(int n, const mlf<N> *A, char op, int tri, const mlf<N> *x, mlf<N> *y, cudaStream_t s) {
    const int g = ceil_div(n, kWarpsPerBlock);
    SDPG_KT_BEGIN(s);
    if ((op == 'T' || op == 't') && n >= 128)
        matvec_t_split_kernel<N><<<ceil_div(n, kWarpsPerBlock / kMvSplit), 32 * kWarpsPerBlock, 0, s>>>(n, A, tri, x, y,
                                                                                                   nullptr);
    else if (op == 'T' || op == 't')
        matvec_t_kernel<N><<<g, 32 * kWarpsPerBlock, 0, s>>>(n, A, tri, x, y);
    else
        matvec_n_kernel<N><<<g, 32 * kWarpsPerBlock, 0, s>>>(n, A, tri, x, y);
    SDPG_CHECK_LAUNCH_KT("matvec_kernel", s);
}

template <int N>
void k_tridiag_min(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status, cudaStream_t s, const int *gate) {
    if (k > kMaxTri) throw sdpg_error(SDPG_ERR_TOO_LARGE, "tridiagonal larger than 512");
    static std::once_flag once;
    std::call_once(once, [] {
        SDPG_CUDA(cudaFuncSetAttribute(tridiag_min_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(2 * kMaxTri * sizeof(mlf<N>))));
    });
    SDPG_KT_BEGIN(s);
    tridiag_min_kernel<N><<<1, 32, (size_t)(2 * k) * sizeof(mlf<N>), s>>>(k, d, e, out, status, gate);
    SDPG_CHECK_LAUNCH_KT("tridiag_min_kernel", s);
}

// ---- Lanczos steps under device control (the loop of Lal::getMinEigen,
// sdpa_linear.cpp:27-124, without a host round trip per step) ----
//
// Per run: slots sl[0] 1/beta, sl[1] beta, sl[4..5] the tridiagonal solver's output
// (lambda, z), sl[6] r.r, sl[8] min, sl[9] min_old, sl[10] error; ctl[0] = 1 while the
// run goes on, ctl[1] = steps done.  Every kernel of a step returns at once when ctl[0]
// is 0, so the host can enqueue several steps ahead and read the state once.

// The next step's vectors, by the CTA that decided to take it: qold = q, q = r / beta.
template <int N>
__device__ void lz_advance(int n, const mlf<N> *r, const mlf<N> *sl, mlf<N> *q, mlf<N> *qold, const int *ctl) {
    if (!ctl[0]) return;
    const mlf<N> inv = sl[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        qold[i] = q[i];
        q[i] = mlc_mul(r[i], inv);
    }
}

template <int N>
__global__ void lz_next_kernel(int n, const mlf<N> *r, const mlf<N> *sl, mlf<N> *q, mlf<N> *qold, const int *ctl) {
    if (!ctl[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    qold[i] = q[i];
    q[i] = ml_mul(r[i], sl[0]);  // q = r / beta
}

// The loop control after step k: the new beta from r.r, the Ritz value of an eigenvalue
// step, and the loop condition for step k + 1 (Lal::getMinEigen's while test), in three
// parts so that an eigenvalue step can form beta beside the tridiagonal solve.

// beta = sqrt(r.r) and 1/beta from one inverse square root: y = (r.r)^(-1/2) is 1/beta,
// beta = (r.r) y refined by half a Newton step; into te[k], sl[1], sl[0]
template <int N>
__device__ mlf<N> lz_beta(mlf<N> *sl, mlf<N> *te, int *ctl, int k) {
    const mlf<N> rr = sl[6];
    const mlf<N> y = mlc_rsqrt(rr);
    mlf<N> beta = mlc_mul(rr, y);
    beta = mlc_add(beta, ml_ldexp(mlc_mul(y, mlc_sub(rr, mlc_mul(beta, beta))), -1));
    if (ml_is_zero(rr) || rr.s) beta = ml_zero<N>();
    te[k] = beta;
    sl[1] = beta;
    sl[0] = ml_is_zero(beta) ? ml_zero<N>() : y;
    ctl[1] = k + 1;
    return beta;
}

// the Ritz value of an eigenvalue step becomes the current minimum, its error term the
// current error
template <int N>
__device__ void lz_ritz(mlf<N> *sl) {
    sl[9] = sl[8];
    sl[8] = sl[4];
    sl[10] = sl[5];
}

// the loop condition for step k + 1
template <int N>
__device__ void lz_go(const mlf<N> *sl, int *ctl, int k, int n, int kgo, int kmax, const mlf<N> &beta) {
    const int kn = k + 1;
    const mlf<N> mn = sl[8], mo = sl[9], er = sl[10];
    bool go = kn < n && kn < kgo && ml_cmp(beta, ml_from_double<N>(1.0e-16)) > 0;
    if (go) {
        const mlf<N> amin = ml_abs(mn);
        const bool c1 = ml_cmp(ml_abs(mlc_sub(mn, mo)),
                               mlc_add(mlc_mul(ml_from_double<N>(1.0e-5), amin), ml_from_double<N>(1.0e-8))) > 0;
        const bool c2 = ml_cmp(ml_abs(mlc_mul(er, beta)),
                               mlc_add(mlc_mul(ml_from_double<N>(1.0e-2), amin), ml_from_double<N>(1.0e-4))) > 0;
        go = c1 || c2;
    }
    if (kn + 1 >= kmax) go = false;
    ctl[0] = go ? 1 : 0;
}

template <int N>
__device__ void lz_control(mlf<N> *sl, mlf<N> *te, int *ctl, int k, int eig, int n, int kgo, int kmax) {
    if (eig) lz_ritz(sl);
    const mlf<N> beta = lz_beta(sl, te, ctl, k);
    lz_go(sl, ctl, k, n, kgo, kmax, beta);
}

// alpha = q.w into td[k] (the first part of an eigenvalue step's update)
template <int N>
__global__ void __launch_bounds__(256) lz_alpha_kernel(int n, const mlf<N> *w, const mlf<N> *q, mlf<N> *td,
                                                       const int *ctl, int k) {
    if (!ctl[0]) return;
    const int stride = blockDim.x;
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
    int i = threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        a0 = mlc_add(a0, mlc_mul(q[i], w[i]));
        a1 = mlc_add(a1, mlc_mul(q[i + stride], w[i + stride]));
    }
    if (i < n) a0 = mlc_add(a0, mlc_mul(q[i], w[i]));
    const mlf<N> alpha = mlc_block_sum(mlc_add(a0, a1));
    if (threadIdx.x == 0) td[k] = alpha;
}

// r = (w - alpha q) - beta qold, r.r and the new beta (the second part, beside the
// tridiagonal solve, which reads td[0..k] and te[0..k-1] only)
template <int N>
__global__ void __launch_bounds__(256) lz_rest_kernel(int n, const mlf<N> *w, const mlf<N> *q, const mlf<N> *qold,
                                                      const mlf<N> *td, mlf<N> *te, mlf<N> *sl, mlf<N> *r, int *ctl,
                                                      int k) {
    if (!ctl[0]) return;
    const int stride = blockDim.x;
    const mlf<N> al = td[k], be = sl[1];
    for (int j = threadIdx.x; j < n; j += stride) r[j] = mlc_sub(mlc_sub(w[j], mlc_mul(q[j], al)), mlc_mul(qold[j], be));
    __syncthreads();
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
    int i = threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        a0 = mlc_add(a0, mlc_mul(r[i], r[i]));
        a1 = mlc_add(a1, mlc_mul(r[i + stride], r[i + stride]));
    }
    if (i < n) a0 = mlc_add(a0, mlc_mul(r[i], r[i]));
    const mlf<N> rr = mlc_block_sum(mlc_add(a0, a1));
    if (threadIdx.x == 0) {
        sl[6] = rr;
        lz_beta(sl, te, ctl, k);
    }
}

// after the tridiagonal solve: the Ritz value, the loop test and the next step's vectors
template <int N>
__global__ void __launch_bounds__(256) lz_decide_kernel(int n, const mlf<N> *r, mlf<N> *q, mlf<N> *qold, mlf<N> *sl,
                                                        int *ctl, int k, int kgo, int kmax) {
    // every thread reads the flag before thread 0 may rewrite it
    const int go = ctl[0];
    __syncthreads();
    if (!go) return;
    if (threadIdx.x == 0) {
        lz_ritz(sl);
        lz_go(sl, ctl, k, n, kgo, kmax, sl[1]);
    }
    __syncthreads();
    lz_advance(n, r, sl, q, qold, ctl);
}

// alpha = q.w (into the tridiagonal's diagonal td[k]), r = (w - alpha q) - beta qold, and
// r.r in one CTA of 256 threads (the strided pairs and block sum of the dot kernel);
// without an eigenvalue solve at this step also the loop control.
template <int N>
__global__ void __launch_bounds__(256) lz_update_kernel(int n, const mlf<N> *w, mlf<N> *q, mlf<N> *qold,
                                                        mlf<N> *td, mlf<N> *te, mlf<N> *sl, mlf<N> *r, int *ctl,
                                                        int k, int eig, int kgo, int kmax) {
    __shared__ mlf<N> alpha_s;
    if (!ctl[0]) return;
    const int stride = blockDim.x;
    mlf<N> a0 = ml_zero<N>(), a1 = ml_zero<N>();
    int i = threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        a0 = mlc_add(a0, mlc_mul(q[i], w[i]));
        a1 = mlc_add(a1, mlc_mul(q[i + stride], w[i + stride]));
    }
    if (i < n) a0 = mlc_add(a0, mlc_mul(q[i], w[i]));
    const mlf<N> alpha = mlc_block_sum(mlc_add(a0, a1));
    if (threadIdx.x == 0) {
        alpha_s = alpha;
        td[k] = alpha;
    }
    __syncthreads();
    const mlf<N> al = alpha_s, be = sl[1];
    for (int j = threadIdx.x; j < n; j += stride) r[j] = mlc_sub(mlc_sub(w[j], mlc_mul(q[j], al)), mlc_mul(qold[j], be));
    __syncthreads();
    a0 = ml_zero<N>();
    a1 = ml_zero<N>();
    i = threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        a0 = mlc_add(a0, mlc_mul(r[i], r[i]));
        a1 = mlc_add(a1, mlc_mul(r[i + stride], r[i + stride]));
    }
    if (i < n) a0 = mlc_add(a0, mlc_mul(r[i], r[i]));
    const mlf<N> rr = mlc_block_sum(mlc_add(a0, a1));
    if (threadIdx.x == 0) {
        sl[6] = rr;
        if (!eig) lz_control(sl, te, ctl, k, 0, n, kgo, kmax);
    }
    if (!eig) {
        __syncthreads();
        lz_advance(n, r, sl, q, qold, ctl);
    }
}

template <int N>
__global__ void __launch_bounds__(256) lz_control_kernel(int n, const mlf<N> *r, mlf<N> *q, mlf<N> *qold, mlf<N> *sl,
                                                         mlf<N> *te, int *ctl, int k, int kgo, int kmax) {
    // every thread reads the flag before thread 0 may rewrite it
    const int go = ctl[0];
    __syncthreads();
    if (!go) return;
    if (threadIdx.x == 0) lz_control(sl, te, ctl, k, 1, n, kgo, kmax);
    __syncthreads();
    lz_advance(n, r, sl, q, qold, ctl);
}

template <int N>
void k_lanczos_step(int n, const mlf<N> *M, mlf<N> *r, mlf<N> *q, mlf<N> *qold, mlf<N> *w, mlf<N> *td, mlf<N> *te,
                    mlf<N> *sl, int *ctl, int *status, int k, int eig, int kgo, int kmax, cudaStream_t s,
                    cudaStream_t side, cudaEvent_t ev_fork, cudaEvent_t ev_join) {
    if (k == 0) {  // later steps get q from the previous step's update or control kernel
        SDPG_KT_BEGIN(s);
        lz_next_kernel<N><<<ceil_div(n, 128), 128, 0, s>>>(n, r, sl, q, qold, ctl);
        SDPG_CHECK_LAUNCH_KT("lz_next_kernel", s);
    }
    if (n >= 128) {
        SDPG_KT_BEGIN(s);
        matvec_t_split_kernel<N><<<ceil_div(n, kWarpsPerBlock / kMvSplit), 32 * kWarpsPerBlock, 0, s>>>(n, M, 0, q, w,
                                                                                                   ctl);
    } else {
        SDPG_KT_BEGIN(s);
        matvec_t_kernel<N><<<ceil_div(n, kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(n, M, 0, q, w, ctl);
    }
    SDPG_CHECK_LAUNCH_KTW("lz_matvec_kernel", s, ((double)n * n + 2.0 * n) * sizeof(mlf<N>));
    if (eig && side) {
        // alpha, then the tridiagonal solve on the side stream beside r, r.r and beta
        SDPG_KT_BEGIN(s);
        lz_alpha_kernel<N><<<1, 256, 0, s>>>(n, w, q, td, ctl, k);
        SDPG_CHECK_LAUNCH_KT("lz_update_kernel", s);
        SDPG_CUDA(cudaEventRecord(ev_fork, s));
        SDPG_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
        k_tridiag_min<N>(k + 1, td, te, sl + 4, status, side, ctl);
        SDPG_KT_BEGIN(s);
        lz_rest_kernel<N><<<1, 256, 0, s>>>(n, w, q, qold, td, te, sl, r, ctl, k);
        SDPG_CHECK_LAUNCH_KT("lz_update_kernel", s);
        SDPG_CUDA(cudaEventRecord(ev_join, side));
        SDPG_CUDA(cudaStreamWaitEvent(s, ev_join, 0));
        SDPG_KT_BEGIN(s);
        lz_decide_kernel<N><<<1, 256, 0, s>>>(n, r, q, qold, sl, ctl, k, kgo, kmax);
        SDPG_CHECK_LAUNCH_KT("lz_control_kernel", s);
        return;
    }
    SDPG_KT_BEGIN(s);
    lz_update_kernel<N><<<1, 256, 0, s>>>(n, w, q, qold, td, te, sl, r, ctl, k, eig, kgo, kmax);
    SDPG_CHECK_LAUNCH_KT("lz_update_kernel", s);
    if (eig) {
        k_tridiag_min<N>(k + 1, td, te, sl + 4, status, s, ctl);
        SDPG_KT_BEGIN(s);
        lz_control_kernel<N><<<1, 256, 0, s>>>(n, r, q, qold, sl, te, ctl, k, kgo, kmax);
        SDPG_CHECK_LAUNCH_KT("lz_control_kernel", s);
    }
}

// The LP rule of Jal::getMinEigen (sdpa_jordan.cpp:79-85): min over k of
// X[k][k] * L[k][k] * L[k][k] for a diagonal block (L its inverse Cholesky factor),
// one CTA; out[0] = the minimum, out[1] = 0 (no Lanczos error term).
template <int N>
__global__ void lp_ratio_min_kernel(int n, const mlf<N> *X, const mlf<N> *L, mlf<N> *out) {
    __shared__ mlf<N> part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mlf<N> best = ml_zero<N>();
    bool have = false;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const size_t kk = (size_t)k + (size_t)n * k;
        const mlf<N> v = ml_mul(ml_mul(X[kk], L[kk]), L[kk]);
        if (!have || ml_cmp(v, best) < 0) best = v;
        have = true;
    }
    // lanes without an entry carry +1e50, the reference's starting minimum
    if (!have) best = ml_from_double<N>(1.0e50);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const mlf<N> o = ml_shfl_xor(best, off);
        if (ml_cmp(o, best) < 0) best = o;
    }
    if (lane == 0) part[warp] = best;
    __syncthreads();
    if (warp == 0) {
        best = lane < (int)(blockDim.x >> 5) ? part[lane] : ml_from_double<N>(1.0e50);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const mlf<N> o = ml_shfl_xor(best, off);
            if (ml_cmp(o, best) < 0) best = o;
        }
        if (lane == 0) {
            out[0] = best;
            out[1] = ml_zero<N>();
        }
    }
}

template <int N>
void k_lp_ratio_min(int n, const mlf<N> *X, const mlf<N> *L, mlf<N> *out, cudaStream_t s) {
    SDPG_KT_BEGIN(s);
    lp_ratio_min_kernel<N><<<1, 256, 0, s>>>(n, X, L, out);
    SDPG_CHECK_LAUNCH_KT("lp_ratio_min_kernel", s);
}

template <int N>
void k_tridiagonalize_small(int n, mlf<N> *A, mlf<N> *d, mlf<N> *e, cudaStream_t s) {
    if (n > 64) throw sdpg_error(SDPG_ERR_TOO_LARGE, "small tridiagonalisation limited to n <= 64");
    SDPG_KT_BEGIN(s);
    tridiagonalize_kernel<N><<<1, 128, 0, s>>>(n, A, d, e);
    SDPG_CHECK_LAUNCH_KT("tridiagonalize_kernel", s);
}

#define SDPG_INST_EIG(N)                                                                                  \
    template void k_matvec<N>(int, const mlf<N> *, char, int, const mlf<N> *, mlf<N> *, cudaStream_t);   \
    template void k_tridiag_min<N>(int, const mlf<N> *, const mlf<N> *, mlf<N> *, int *, cudaStream_t,     \
                                   const int *);                                                          \
    template void k_lanczos_step<N>(int, const mlf<N> *, mlf<N> *, mlf<N> *, mlf<N> *, mlf<N> *, mlf<N> *, \
                                    mlf<N> *, mlf<N> *, int *, int *, int, int, int, int, cudaStream_t,    \
                                    cudaStream_t, cudaEvent_t, cudaEvent_t);                               \
    template void k_tridiagonalize_small<N>(int, mlf<N> *, mlf<N> *, mlf<N> *, cudaStream_t);              \
    template void k_lp_ratio_min<N>(int, const mlf<N> *, const mlf<N> *, mlf<N> *, cudaStream_t);
SDPG_INST_EIG(8)
SDPG_INST_EIG(16)

}  // namespace sdpg
