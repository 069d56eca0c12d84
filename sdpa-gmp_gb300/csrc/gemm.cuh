// Block-floating-point multi-limb GEMM (the GPU replacement of the reference's
// Rgemm family, mplapack/Rgemm_omp.cpp:41-127 and Rgemm_{NN,NT,TN,TT}_omp.cpp).
//
//   C = alpha * op(A) * op(B) + beta * C     (column-major, optionally batched)
//
// Method.  Every row i of op(A) gets one exponent EA_i = max_k exponent(a_ik)
// and every column j of op(B) one exponent EB_j.  Each entry becomes the
// integer trunc(a_ik * 2^(R - EA_i)), |.| < 2^R, stored as D balanced
// radix-2^28 digits in [-2^27, 2^27] (int32).  A digit product is then one
// signed 32x32->64 multiply-add (IMAD.WIDE) into an int64 column accumulator.
// Columns below D-1 of each digit product are dropped (truncation error below
// 2^-(28D-6) of max|a_i.| * max|b_.j| per product); every CH k-steps the
// column accumulators are carry-normalised so they never overflow.  The
// epilogue turns the exact column sums back into an mlf, scales by alpha and
// adds beta * C.
//
// Accuracy: |error(c_ij)| <= K * 2^-(R-2) * 2^(EA_i + EB_j), i.e. a normwise
// (row-max x column-max) bound with R = 28D - 2 >= 32N + 22 guard bits; GMP's
// sequential truncated summation in Rgemm has the same form with 2^-p.
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace sdpg {

template <int N>
struct Bfp {
    static constexpr int D = (32 * N + 24 + 27) / 28;  // digits: N=8 -> 10, N=16 -> 20
    static constexpr int R = 28 * D - 2;               // integer magnitude bound 2^R
    static constexpr int C0 = D - 1;                   // lowest kept product column
    static constexpr int NC = D + 2;                   // kept columns C0 .. 2D
    static constexpr int CH = (D <= 12) ? 32 : 16;     // k-steps between carry normalisations
};

// One operand of a GEMM: element (o, k) of op(X) lives at X[b*sb + o*so + k*sk].
template <int N>
struct Operand {
    const mlf<N> *X;
    long long so, sk, sb;
};

template <int N>
struct GemmProblem {
    int M, Nn, K, batch;
    Operand<N> A;  // op(A): M x K, outer index i
    Operand<N> B;  // op(B): K x Nn, outer index j
    mlf<N> *C;
    long long ldc, sc;
    mlf<N> alpha, beta;
    int lower_only;  // 1: only entries with i >= j are written (SYRK-style update)
    // device word set non-zero when a tensor-core kernel of this product gives up a
    // bounded wait (null: the workspace's word, else only the device-wide flag)
    int *error = nullptr;
    // optional: events recorded immediately before / after the digit-GEMM kernel launch
    cudaEvent_t ev_before = nullptr, ev_after = nullptr;
};

// Build operands from BLAS-style (trans, pointer, ld, batch stride) arguments.
template <int N>
inline Operand<N> operand_A(char trans, const mlf<N> *A, long long lda, long long sA) {
    // op(A)[i,k] = A[i + k*lda] ('N') or A[k + i*lda] ('T')
    if (trans == 'N' || trans == 'n') return Operand<N>{A, 1, lda, sA};
    return Operand<N>{A, lda, 1, sA};
}
template <int N>
inline Operand<N> operand_B(char trans, const mlf<N> *B, long long ldb, long long sB) {
    // op(B)[k,j] = B[k + j*ldb] ('N') or B[j + k*ldb] ('T')
    if (trans == 'N' || trans == 'n') return Operand<N>{B, ldb, 1, sB};
    return Operand<N>{B, 1, ldb, sB};
}

// Workspace bytes ml_gemm needs for this problem (for whichever method it selects).
template <int N>
size_t gemm_workspace_bytes(const GemmProblem<N> &p);

// Runs the GEMM on `stream`; scratch is carved from ws (which must already hold
// gemm_workspace_bytes(p) beyond ws.used).  256-bit products with K <= 16384 that are
// not tiny go through the residue-number-system path on the tensor cores
// (crt_gemm.cu); everything else through the digit GEMM below.
template <int N>
void ml_gemm(const GemmProblem<N> &p, Workspace &ws, cudaStream_t stream);

// The digit GEMM alone, with caller-provided scratch of at least
// gemm_bfp_workspace_bytes(p) bytes.
template <int N>
size_t gemm_bfp_workspace_bytes(const GemmProblem<N> &p);
template <int N>
void ml_gemm_scratch(const GemmProblem<N> &p, void *scratch, cudaStream_t stream);

// Residue-number-system path (crt_gemm.cu).
extern int g_gemm_method;  // 0: residue path where it applies, 1: digit GEMM only, 2: residue path always
template <int N>
bool crt_gemm_applies(const GemmProblem<N> &p);
template <int N>
size_t crt_gemm_workspace_bytes(const GemmProblem<N> &p);
template <int N>
void crt_gemm(const GemmProblem<N> &p, void *scratch, cudaStream_t stream);
// Residues of a Cholesky factor's finished columns, kept across its panels (crt_gemm.cu):
// Q planes [kCrtL][rows][kpitch] (row i, column k of the factor), the row scales E and the
// result planes of one panel product.
struct CrtCache {
    __half *Q = nullptr;
    uint16_t *Y = nullptr;
    int *E = nullptr;
    int n = 0, rows = 0, kpitch = 0;
};
size_t crt_cache_bytes(int n);
template <int N>
bool crt_cache_applies(int n);
// zeroes the planes and sets the row scales from A's diagonal (before the factorisation)
template <int N>
CrtCache crt_cache_init(int n, const mlf<N> *A, long long lda, void *mem, cudaStream_t s);
// residues of the finished columns k0 .. k0 + kb - 1 (rows k0 .. n - 1; the diagonal
// block's upper part read as zero)
template <int N>
void crt_cache_put(const CrtCache &c, const mlf<N> *A, long long lda, int k0, int kb, int *error, cudaStream_t s);
// A[k0:n, k0:k0+kb] -= L[k0:n, :kend] L[k0:k0+kb, :kend]^T (lower part of the top block)
// from the cached residues of columns 0 .. kend - 1 (kend <= k0; later columns are not read)
template <int N>
void crt_cache_panel(const CrtCache &c, int k0, int kb, int kend, mlf<N> *A, long long lda, int *error,
                     cudaStream_t s);

// Device-wide sticky flag: set (and never cleared) when any tensor-core kernel on the
// current device gave up a bounded wait, in addition to the product's own error word.
int *crt_error_word();

}  // namespace sdpg
