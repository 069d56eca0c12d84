// C ABI: number-format utilities and the standalone multi-limb GEMM entry
// points.  Every function returns 0 on success or a negative SDPG_ERR_* code;
// sdpg_last_error() gives the message of the calling thread's last failure.
#include <string.h>

#include <string>

#include "capi_util.cuh"
#include "gemm.cuh"
#include "kernels.cuh"
#include "ml_host.h"
#include "sdpg.h"

using namespace sdpg;

namespace sdpg {
thread_local std::string g_last_error;
void set_last_error(const std::string &m) { g_last_error = m; }
}  // namespace sdpg

extern "C" {

const char *sdpg_last_error(void) { return g_last_error.c_str(); }

int sdpg_version(void) { return SDPG_VERSION; }

int sdpg_limbs_for_precision(int precision_bits) {
    if (precision_bits <= 0) return SDPG_ERR_ARG;
    if (precision_bits <= 256) return 8;
    if (precision_bits <= 512) return 16;
    set_last_error("precision above 512 bits is not supported");
    return SDPG_ERR_ARG;
}

int sdpg_ml_elem_bytes(int limbs) {
    if (limbs != 8 && limbs != 16) return SDPG_ERR_ARG;
    return 8 + 4 * limbs;
}

int sdpg_ml_parse(int limbs, const char *text, void *out) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> v;
            if (!ml_parse<N>(text, &v)) throw sdpg_error(SDPG_ERR_ARG, "not a number");
            memcpy(out, &v, sizeof v);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_format(int limbs, const void *v, int digits, char *buf, int cap) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> x;
            memcpy(&x, v, sizeof x);
            std::string s = ml_format_e<N>(x, digits > 0 ? digits - 1 : 0);
            if ((int)s.size() + 1 > cap) throw sdpg_error(SDPG_ERR_ARG, "buffer too small");
            memcpy(buf, s.c_str(), s.size() + 1);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_format_gmp(int limbs, const void *v, const char *fmt, char *buf, int cap) {
    return sdpg_guard([&] {
        if (!v || !fmt || !buf) throw sdpg_error(SDPG_ERR_ARG, "null argument");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> x;
            memcpy(&x, v, sizeof x);
            const std::string s = ml_format_gmp<N>(fmt, x);
            if ((int)s.size() + 1 > cap) throw sdpg_error(SDPG_ERR_ARG, "buffer too small");
            memcpy(buf, s.c_str(), s.size() + 1);
            return (int)s.size();
        });
    });
}

int sdpg_ml_from_double(int limbs, const double *x, long long n, void *out) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> *o = (mlf<N> *)out;
            for (long long i = 0; i < n; ++i) o[i] = ml_from_double<N>(x[i]);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_to_double(int limbs, const void *v, long long n, double *out) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            const mlf<N> *a = (const mlf<N> *)v;
            for (long long i = 0; i < n; ++i) out[i] = ml_to_double<N>(a[i]);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_from_mpf(int limbs, const sdpg_mpf_t *src, long long n, void *out) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> *o = (mlf<N> *)out;
            for (long long i = 0; i < n; ++i) o[i] = ml_from_mpf<N>(src[i]._mp_size, src[i]._mp_exp, src[i]._mp_d);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_to_mpf(int limbs, const void *v, long long n, sdpg_mpf_t *dst) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            const mlf<N> *a = (const mlf<N> *)v;
            for (long long i = 0; i < n; ++i) {
                long ex = 0;
                const int cap = dst[i]._mp_prec + 1;
                dst[i]._mp_size = ml_to_mpf<N>(a[i], &ex, dst[i]._mp_d, cap);
                dst[i]._mp_exp = ex;
            }
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_host_op(int limbs, int op, long long n, const void *a, const void *b, void *out) {
    return sdpg_guard([&] {
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            const mlf<N> *x = (const mlf<N> *)a;
            const mlf<N> *y = (const mlf<N> *)b;
            mlf<N> *o = (mlf<N> *)out;
            for (long long i = 0; i < n; ++i) {
                switch (op) {
                    case SDPG_OP_ADD: o[i] = ml_add(x[i], y[i]); break;
                    case SDPG_OP_SUB: o[i] = ml_sub(x[i], y[i]); break;
                    case SDPG_OP_MUL: o[i] = ml_mul(x[i], y[i]); break;
                    case SDPG_OP_DIV:
                        if (ml_is_zero(y[i])) throw sdpg_error(SDPG_ERR_ARG, "division by zero");
                        o[i] = ml_div(x[i], y[i]);
                        break;
                    case SDPG_OP_SQRT:
                        if (x[i].s && !ml_is_zero(x[i])) throw sdpg_error(SDPG_ERR_ARG, "sqrt of negative");
                        o[i] = ml_sqrt(x[i]);
                        break;
                    default: throw sdpg_error(SDPG_ERR_ARG, "unknown op");
                }
            }
            return (int)SDPG_OK;
        });
    });
}

int sdpg_ml_compare(int limbs, const void *a, const void *b, int *result) {
    return sdpg_guard([&] {
        if (!a || !b || !result) throw sdpg_error(SDPG_ERR_ARG, "null operand");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            mlf<N> x, y;
            memcpy(&x, a, sizeof x);
            memcpy(&y, b, sizeof y);
            const int c = ml_cmp(x, y);
            *result = c < 0 ? -1 : c > 0 ? 1 : 0;
            return (int)SDPG_OK;
        });
    });
}

int sdpg_rgemm_device(int limbs, char transa, char transb, int m, int n, int k, const void *alpha,
                      const void *A, int lda, const void *B, int ldb, const void *beta, void *C, int ldc,
                      void *stream) {
    return sdpg_guard([&] {
        if (m < 0 || n < 0 || k < 0) throw sdpg_error(SDPG_ERR_ARG, "negative dimension");
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
            Workspace &ws = thread_workspace((cudaStream_t)stream);
            ws.reset();
            ws.reserve(gemm_workspace_bytes(p) + 512);
            ml_gemm<N>(p, ws, (cudaStream_t)stream);
            return (int)SDPG_OK;
        });
    });
}

int sdpg_rgemm(int limbs, char transa, char transb, int m, int n, int k, const void *alpha, const void *A,
               int lda, const void *B, int ldb, const void *beta, void *C, int ldc) {
    return sdpg_guard([&] {
        const int eb = sdpg_ml_elem_bytes(limbs);
        if (eb < 0) throw sdpg_error(SDPG_ERR_ARG, "unsupported limb count");
        const bool ta = (transa == 'T' || transa == 't' || transa == 'C' || transa == 'c');
        const bool tb = (transb == 'T' || transb == 't' || transb == 'C' || transb == 'c');
        const size_t na = (size_t)lda * (ta ? m : k), nb = (size_t)ldb * (tb ? k : n), nc = (size_t)ldc * n;
        DeviceBuffer dA(na * eb), dB(nb * eb), dC(nc * eb);
        SDPG_CUDA(cudaMemcpy(dA.p, A, na * eb, cudaMemcpyHostToDevice));
        SDPG_CUDA(cudaMemcpy(dB.p, B, nb * eb, cudaMemcpyHostToDevice));
        SDPG_CUDA(cudaMemcpy(dC.p, C, nc * eb, cudaMemcpyHostToDevice));
        int rc = sdpg_rgemm_device(limbs, transa, transb, m, n, k, alpha, dA.p, lda, dB.p, ldb, beta, dC.p, ldc,
                                   nullptr);
        if (rc != SDPG_OK) return rc;
        SDPG_CUDA(cudaMemcpy(C, dC.p, nc * eb, cudaMemcpyDeviceToHost));
        return (int)SDPG_OK;
    });
}

}  // extern "C"

namespace {

template <class F>
int with_device_copy(int limbs, size_t count, const void *host, bool copy_back, void *host_out, F &&f) {
    const int eb = 8 + 4 * limbs;
    DeviceBuffer d(count * eb > 0 ? count * eb : 16);
    if (count) SDPG_CUDA(cudaMemcpy(d.p, host, count * eb, cudaMemcpyHostToDevice));
    int rc = f(d.p);
    SDPG_CUDA(cudaDeviceSynchronize());
    if (copy_back && count) SDPG_CUDA(cudaMemcpy(host_out, d.p, count * eb, cudaMemcpyDeviceToHost));
    return rc;
}

}  // namespace

extern "C" {

int sdpg_rpotrf(int limbs, int n, void *A, int lda, int *info) {
    return sdpg_guard([&] {
        if (n < 0 || lda < (n > 1 ? n : 1) || !A || !info) throw sdpg_error(SDPG_ERR_ARG, "bad arguments");
        if (n == 0) {
            *info = 0;
            return (int)SDPG_OK;
        }
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            DeviceBuffer dinfo(sizeof(int));
            int rc = with_device_copy(limbs, (size_t)lda * n, A, true, A, [&](void *dA) {
                Workspace &ws = thread_workspace(nullptr);
                ws.reset();
                ws.reserve(ml_potrf_workspace_bytes<N>(n) + (1 << 20));
                ml_potrf<N>(n, (mlf<N> *)dA, lda, (int *)dinfo.p, ws, nullptr);
                return (int)SDPG_OK;
            });
            SDPG_CUDA(cudaMemcpy(info, dinfo.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (*info == -1) throw sdpg_error(SDPG_ERR_TIMEOUT, "Cholesky panel: a bounded wait timed out");
            return rc;
        });
    });
}

int sdpg_inv_lower(int limbs, int n, const void *L, int ldl, void *Linv) {
    return sdpg_guard([&] {
        if (n <= 0 || ldl < n || !L || !Linv) throw sdpg_error(SDPG_ERR_ARG, "bad arguments");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            DeviceBuffer dout((size_t)n * n * sizeof(mlf<N>));
            int rc = with_device_copy(limbs, (size_t)ldl * n, L, false, nullptr, [&](void *dL) {
                Workspace &ws = thread_workspace(nullptr);
                ws.reset();
                ws.reserve(ml_trtri_workspace_bytes<N>(n) + (1 << 20));
                ml_trtri_lower<N>(n, (const mlf<N> *)dL, ldl, (mlf<N> *)dout.p, ws, nullptr);
                return (int)SDPG_OK;
            });
            SDPG_CUDA(cudaMemcpy(Linv, dout.p, (size_t)n * n * sizeof(mlf<N>), cudaMemcpyDeviceToHost));
            return rc;
        });
    });
}

int sdpg_solve_systems(int limbs, int n, const void *L, int ldl, void *x) {
    return sdpg_guard([&] {
        if (n <= 0 || ldl < n || !L || !x) throw sdpg_error(SDPG_ERR_ARG, "bad arguments");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            DeviceBuffer dx((size_t)n * sizeof(mlf<N>));
            SDPG_CUDA(cudaMemcpy(dx.p, x, (size_t)n * sizeof(mlf<N>), cudaMemcpyHostToDevice));
            int rc = with_device_copy(limbs, (size_t)ldl * n, L, false, nullptr, [&](void *dL) {
                Workspace &ws = thread_workspace(nullptr);
                ws.reset();
                ws.reserve(ml_potrs_prepare_bytes<N>(n) + (1 << 20));
                mlf<N> *Dinv = (mlf<N> *)ws.carve(ml_potrs_prepare_bytes<N>(n));
                ml_potrs_prepare<N>(n, (const mlf<N> *)dL, ldl, Dinv, nullptr);
                ml_potrs_solve<N>(n, (const mlf<N> *)dL, ldl, Dinv, (mlf<N> *)dx.p, nullptr);
                int st = 0;
                SDPG_CUDA(cudaMemcpy(&st, ml_potrs_status<N>(n, Dinv), sizeof(int), cudaMemcpyDeviceToHost));
                if (st != 0) throw sdpg_error(SDPG_ERR_TIMEOUT, "triangular solve: a bounded wait timed out");
                return (int)SDPG_OK;
            });
            SDPG_CUDA(cudaMemcpy(x, dx.p, (size_t)n * sizeof(mlf<N>), cudaMemcpyDeviceToHost));
            return rc;
        });
    });
}

int sdpg_tridiag_min(int limbs, int k, const void *d, const void *e, void *out2) {
    return sdpg_guard([&] {
        if (k <= 0 || !d || !out2 || (k > 1 && !e)) throw sdpg_error(SDPG_ERR_ARG, "bad arguments");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            const size_t eb = sizeof(mlf<N>);
            DeviceBuffer dd(k * eb), de((k > 1 ? k - 1 : 1) * eb), dout(2 * eb), dst(sizeof(int));
            SDPG_CUDA(cudaMemcpy(dd.p, d, k * eb, cudaMemcpyHostToDevice));
            if (k > 1) SDPG_CUDA(cudaMemcpy(de.p, e, (k - 1) * eb, cudaMemcpyHostToDevice));
            k_tridiag_min<N>(k, (const mlf<N> *)dd.p, (const mlf<N> *)de.p, (mlf<N> *)dout.p, (int *)dst.p, nullptr);
            SDPG_CUDA(cudaDeviceSynchronize());
            int st = 0;
            SDPG_CUDA(cudaMemcpy(&st, dst.p, sizeof(int), cudaMemcpyDeviceToHost));
            SDPG_CUDA(cudaMemcpy(out2, dout.p, 2 * eb, cudaMemcpyDeviceToHost));
            if (st != 0) throw sdpg_error(SDPG_ERR_NOCONV, "tridiagonal eigenvalue iteration did not converge");
            return (int)SDPG_OK;
        });
    });
}

int sdpg_sym_min_eigen(int limbs, int n, const void *A, void *out) {
    return sdpg_guard([&] {
        if (n <= 0 || n > 64 || !A || !out) throw sdpg_error(SDPG_ERR_ARG, "n must be in 1..64");
        return dispatch_limbs(limbs, [&](auto tag) {
            constexpr int N = decltype(tag)::value;
            const size_t eb = sizeof(mlf<N>);
            DeviceBuffer dA((size_t)n * n * eb), dd(n * eb), de(n * eb), dout(2 * eb), dst(sizeof(int));
            SDPG_CUDA(cudaMemcpy(dA.p, A, (size_t)n * n * eb, cudaMemcpyHostToDevice));
            k_tridiagonalize_small<N>(n, (mlf<N> *)dA.p, (mlf<N> *)dd.p, (mlf<N> *)de.p, nullptr);
            k_tridiag_min<N>(n, (const mlf<N> *)dd.p, (const mlf<N> *)de.p, (mlf<N> *)dout.p, (int *)dst.p, nullptr);
            SDPG_CUDA(cudaDeviceSynchronize());
            int st = 0;
            SDPG_CUDA(cudaMemcpy(&st, dst.p, sizeof(int), cudaMemcpyDeviceToHost));
            SDPG_CUDA(cudaMemcpy(out, dout.p, eb, cudaMemcpyDeviceToHost));
            if (st != 0) throw sdpg_error(SDPG_ERR_NOCONV, "smallest eigenvalue: Newton iteration did not converge");
            return (int)SDPG_OK;
        });
    });
}

}  // extern "C"
