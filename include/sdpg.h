/* sdpg.h -- C ABI of the GB300 multi-limb SDPA Newton-step library (libsdpg.so).
 *
 * The reference (SDPA-GMP 7.1.3) has no plugin or FFI layer: its hot path is
 * reached through C++ classes inside one binary (Newton, Lal, Jal in
 * sdpa_newton.h, sdpa_linear.h, sdpa_jordan.h, over the containers of
 * sdpa_struct.h).  Each entry point below names the reference function it
 * replaces.  Conventions:
 *
 *   - every function returns 0 (SDPG_OK) or a negative SDPG_ERR_* code and
 *     never throws; sdpg_last_error() returns the calling thread's message;
 *   - numbers cross the boundary in one of three forms:
 *       * "ml" arrays: the library's own element layout, `limbs` 32-bit limbs
 *         per value: { int32 e; uint32 s; uint32 m[limbs]; }, value =
 *         (-1)^s * (sum_k m[k] 2^(32k)) * 2^(e - 32*limbs), m normalised
 *         (top bit of m[limbs-1] set) or all zero; 8 + 4*limbs bytes each;
 *       * sdpg_mpf_t arrays, layout-identical to GMP's __mpf_struct, so an
 *         array of mpf_class (one mpf_t member each) can be passed directly;
 *       * decimal text (the .dat-s reader) or doubles (exact conversion);
 *   - limbs is 8 (256-bit mantissa) or 16 (512-bit); sdpg_limbs_for_precision
 *     maps a param.sdpa precision to it;
 *   - matrices are column-major (the reference's de_ele[i + nRow*j],
 *     sdpa_struct.h:111-133);
 *   - "host" entry points take host buffers and do the copies; "_device"
 *     variants take device pointers and an optional cudaStream_t (NULL =
 *     default stream) and do not synchronise.
 */
#ifndef SDPG_H
#define SDPG_H

#ifdef __cplusplus
extern "C" {
#endif

#define SDPG_VERSION 100

enum {
    SDPG_OK = 0,
    SDPG_ERR_ARG = -1,
    SDPG_ERR_CUDA = -2,
    SDPG_ERR_NOT_PD = -3,
    SDPG_ERR_NOCONV = -4,
    SDPG_ERR_IO = -5,
    SDPG_ERR_STATE = -6,
    SDPG_ERR_TOO_LARGE = -7,
    SDPG_ERR_TIMEOUT = -8
};

enum { SDPG_OP_ADD = 0, SDPG_OP_SUB = 1, SDPG_OP_MUL = 2, SDPG_OP_DIV = 3, SDPG_OP_SQRT = 4 };

/* GMP's public float struct (gmp.h, __mpf_struct) on an LP64 64-bit-limb build. */
typedef struct {
    int _mp_prec;
    int _mp_size;
    long _mp_exp;
    unsigned long *_mp_d;
} sdpg_mpf_t;

const char *sdpg_last_error(void);
int sdpg_version(void);

/* precision bits (param.sdpa line 11, sdpa_parts.cpp:198) -> limbs (8 or 16) */
int sdpg_limbs_for_precision(int precision_bits);
int sdpg_ml_elem_bytes(int limbs);

/* Number conversions (the reference reads numbers with gmp_fscanf "%Fe",
 * sdpa_io.cpp:138-142, and prints them with gmp_fprintf, sdpa_io.cpp:1086-1162). */
int sdpg_ml_parse(int limbs, const char *text, void *out);
int sdpg_ml_format(int limbs, const void *v, int digits, char *buf, int cap);
int sdpg_ml_from_double(int limbs, const double *x, long long n, void *out);
int sdpg_ml_to_double(int limbs, const void *v, long long n, double *out);
int sdpg_ml_from_mpf(int limbs, const sdpg_mpf_t *src, long long n, void *out);
/* dst[i]._mp_d must hold _mp_prec + 1 limbs (as GMP allocates). */
int sdpg_ml_to_mpf(int limbs, const void *v, long long n, sdpg_mpf_t *dst);
/* Elementwise host arithmetic in the ml format (SDPG_OP_*); b is ignored for SQRT. */
int sdpg_ml_host_op(int limbs, int op, long long n, const void *a, const void *b, void *out);

/* C = alpha*op(A)*op(B) + beta*C  -- replaces Rgemm (mplapack/Rgemm_omp.cpp:41-127,
 * dispatching to Rgemm_{NN,NT,TN,TT}_omp.cpp) as called by Lal::multiply
 * (sdpa_linear.cpp:856-875).  transa/transb: 'N' or 'T'. */
int sdpg_rgemm(int limbs, char transa, char transb, int m, int n, int k, const void *alpha, const void *A,
               int lda, const void *B, int ldb, const void *beta, void *C, int ldc);
int sdpg_rgemm_device(int limbs, char transa, char transb, int m, int n, int k, const void *alpha,
                      const void *A, int lda, const void *B, int ldb, const void *beta, void *C, int ldc,
                      void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SDPG_H */
