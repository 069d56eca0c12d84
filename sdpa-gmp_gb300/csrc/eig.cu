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

#include <climits>

#include "kernels.cuh"
#include "mlwarp.cuh"

namespace sdpg {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxTri = 512;

// y[o] = sum_i A[i,o] x[i]  (op 'T': columns of A), tri: 0 all rows, 1 rows i >= o, 2 rows i <= o
template <int N>
__global__ void matvec_t_kernel(int n, const mlf<N> *A, int tri, const mlf<N> *x, mlf<N> *y) {
    const int o = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (o >= n) return;
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

template <int N>
__global__ void lanczos_update_kernel(int n, const mlf<N> *w, const mlf<N> *q, const mlf<N> *qold,
                                      const mlf<N> *alpha, const mlf<N> *beta, mlf<N> *r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // r = w - q*alpha; r = r - qold*beta   (Lal::let(r,'=',w,'-',q,&alpha) then (r,'-',qold,&beta))
    mlf<N> t = ml_sub(w[i], ml_mul(q[i], *alpha));
    r[i] = ml_sub(t, ml_mul(qold[i], *beta));
}

template <int N>
__global__ void lanczos_next_kernel(int n, const mlf<N> *r, const mlf<N> *rbeta, mlf<N> *q, mlf<N> *qold) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    qold[i] = q[i];
    q[i] = ml_mul(r[i], *rbeta);
}

__device__ int sturm_count_d(int k, const double *d, const double *e2, double x) {
    int cnt = 0;
    double q = d[0] - x;
    if (q < 0) ++cnt;
    for (int i = 1; i < k; ++i) {
        if (q == 0.0) q = -DBL_EPSILON * (fabs(d[i - 1]) + 1e-300);
        q = d[i] - x - e2[i - 1] / q;
        if (q < 0) ++cnt;
    }
    return cnt;
}

// p_k(lam) and p_k'(lam), p_{k-1}(lam) by the monic three-term recurrence
template <int N>
__device__ void charpoly(int k, const mlf<N> *d, const mlf<N> *e, const mlf<N> &lam, mlf<N> *pk, mlf<N> *dpk,
                         mlf<N> *pkm1) {
    mlf<N> p_prev = ml_one<N>(), p_cur = ml_sub(lam, d[0]);
    mlf<N> dp_prev = ml_zero<N>(), dp_cur = ml_one<N>();
    for (int i = 1; i < k; ++i) {
        const mlf<N> a = ml_sub(lam, d[i]);
        const mlf<N> b2 = ml_mul(e[i - 1], e[i - 1]);
        const mlf<N> p_new = ml_sub(ml_mul(a, p_cur), ml_mul(b2, p_prev));
        const mlf<N> dp_new = ml_sub(ml_add(p_cur, ml_mul(a, dp_cur)), ml_mul(b2, dp_prev));
        p_prev = p_cur;
        p_cur = p_new;
        dp_prev = dp_cur;
        dp_cur = dp_new;
    }
    *pk = p_cur;
    *dpk = dp_cur;
    *pkm1 = p_prev;
}

template <int N>
__global__ void tridiag_min_kernel(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (k <= 0 || k > kMaxTri) {
        *status = 1;
        return;
    }
    if (k == 1) {
        out[0] = d[0];
        out[1] = ml_one<N>();
        *status = 0;
        return;
    }
    double dd[kMaxTri], e2[kMaxTri];
    double lo = 0, hi = 0;
    for (int i = 0; i < k; ++i) {
        dd[i] = ml_to_double(d[i]);
        const double ea = (i > 0 ? fabs(ml_to_double(e[i - 1])) : 0.0) + (i + 1 < k ? fabs(ml_to_double(e[i])) : 0.0);
        if (i + 1 < k) {
            const double ev = ml_to_double(e[i]);
            e2[i] = ev * ev;
        }
        const double l = dd[i] - ea, h = dd[i] + ea;
        if (i == 0 || l < lo) lo = l;
        if (i == 0 || h > hi) hi = h;
    }
    // bisection for the smallest eigenvalue: count(x) >= 1 means x above it
    double a = lo - 1e-300 - fabs(lo) * 1e-15, b = hi + fabs(hi) * 1e-15 + 1e-300;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (a + b);
        if (mid <= a || mid >= b) break;
        if (sturm_count_d(k, dd, e2, mid) >= 1) b = mid;
        else a = mid;
    }
    mlf<N> lam = ml_from_double<N>(0.5 * (a + b));
    // Newton on the characteristic polynomial.  Converged when the step is below
    // 2^-(32N+2) of the matrix scale S = max(|lo|, |hi|) (the Gershgorin bound), or
    // once steps stop shrinking (the rounding floor of the recurrence is reached).
    const int scale_e = ml_from_double<N>(fmax(fabs(lo), fabs(hi))).e;
    mlf<N> pk, dpk, pkm1;
    int st = 2;  // not converged
    int prev_e = INT_MAX;
    for (int it = 0; it < 16; ++it) {
        charpoly<N>(k, d, e, lam, &pk, &dpk, &pkm1);
        if (ml_is_zero(pk)) {
            st = 0;
            break;
        }
        if (ml_is_zero(dpk)) break;
        const mlf<N> delta = ml_div(pk, dpk);
        lam = ml_sub(lam, delta);
        if (ml_is_zero(delta) || delta.e < scale_e - (32 * N + 2) ||
            (!ml_is_zero(lam) && delta.e < lam.e - (32 * N + 2)) || (it >= 2 && delta.e > prev_e - 2)) {
            st = 0;
            charpoly<N>(k, d, e, lam, &pk, &dpk, &pkm1);
            break;
        }
        prev_e = delta.e;
    }
    out[0] = lam;
    // z^2 = p_{k-1}(lam) / p_k'(lam)  (>= 0 at a simple root)
    mlf<N> z2 = ml_is_zero(dpk) ? ml_zero<N>() : ml_div(pkm1, dpk);
    z2 = ml_abs(z2);
    out[1] = ml_sqrt(z2);
    *status = st;
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
    if (op == 'T' || op == 't') matvec_t_kernel<N><<<g, 32 * kWarpsPerBlock, 0, s>>>(n, A, tri, x, y);
    else matvec_n_kernel<N><<<g, 32 * kWarpsPerBlock, 0, s>>>(n, A, tri, x, y);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void k_lanczos_update(int n, const mlf<N> *w, const mlf<N> *q, const mlf<N> *qold, const mlf<N> *alpha,
                      const mlf<N> *beta, mlf<N> *r, cudaStream_t s) {
    lanczos_update_kernel<N><<<ceil_div(n, 128), 128, 0, s>>>(n, w, q, qold, alpha, beta, r);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void k_lanczos_next(int n, const mlf<N> *r, const mlf<N> *beta, mlf<N> *q, mlf<N> *qold, cudaStream_t s) {
    lanczos_next_kernel<N><<<ceil_div(n, 128), 128, 0, s>>>(n, r, beta, q, qold);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void k_tridiag_min(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status, cudaStream_t s) {
    if (k > kMaxTri) throw sdpg_error(SDPG_ERR_TOO_LARGE, "tridiagonal larger than 512");
    tridiag_min_kernel<N><<<1, 32, 0, s>>>(k, d, e, out, status);
    SDPG_CHECK_LAUNCH();
}

template <int N>
void k_tridiagonalize_small(int n, mlf<N> *A, mlf<N> *d, mlf<N> *e, cudaStream_t s) {
    if (n > 64) throw sdpg_error(SDPG_ERR_TOO_LARGE, "small tridiagonalisation limited to n <= 64");
    tridiagonalize_kernel<N><<<1, 128, 0, s>>>(n, A, d, e);
    SDPG_CHECK_LAUNCH();
}

#define SDPG_INST_EIG(N)                                                                                  \
    template void k_matvec<N>(int, const mlf<N> *, char, int, const mlf<N> *, mlf<N> *, cudaStream_t);   \
    template void k_lanczos_update<N>(int, const mlf<N> *, const mlf<N> *, const mlf<N> *, const mlf<N> *, \
                                      const mlf<N> *, mlf<N> *, cudaStream_t);                            \
    template void k_lanczos_next<N>(int, const mlf<N> *, const mlf<N> *, mlf<N> *, mlf<N> *, cudaStream_t); \
    template void k_tridiag_min<N>(int, const mlf<N> *, const mlf<N> *, mlf<N> *, int *, cudaStream_t);  \
    template void k_tridiagonalize_small<N>(int, mlf<N> *, mlf<N> *, mlf<N> *, cudaStream_t);
SDPG_INST_EIG(8)
SDPG_INST_EIG(16)

}  // namespace sdpg
