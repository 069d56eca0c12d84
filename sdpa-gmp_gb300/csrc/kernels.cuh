// Host launchers of the dense / constraint / factorisation / eigen kernels.
// All take device pointers and a stream; matrices are column-major n x n
// mlf<N> blocks (the reference's DenseMatrix de_ele[i + nRow*j]).
#pragma once
#include "common.cuh"
#include "gemm.cuh"

namespace sdpg {

// Constraint matrices restricted to one SDP block, device side.
//   * sparse constraints: COO with the symmetric expansion ((i,j) and (j,i) for
//     i != j, duplicates merged), so A.M = sum v*M[r,c] for any M;
//   * dense constraints: full n x n matrices in `dense`.
template <int N>
struct BlockDev {
    int n = 0;        // block size
    int nc = 0;       // constraints touching the block
    int ndense = 0;   // how many of them are dense
    int *cid = nullptr;      // [nc] global constraint index
    int *rank = nullptr;     // [nc] rank in (NonZeroEffect, index) order
    int *formula = nullptr;  // [nc] 0 = F1, 1 = F2, 2 = F3
    int *sp_off = nullptr;   // [nc+1] COO offsets (dense constraints: empty range)
    int *sp_row = nullptr, *sp_col = nullptr;
    mlf<N> *sp_val = nullptr;
    int *dn_slot = nullptr;  // [nc] slot in `dense` or -1
    int *dn_cid = nullptr;   // [ndense] global constraint index of each dense slot
    int *dn_local = nullptr; // [ndense] local index of each dense slot
    long long *dn_off = nullptr;  // [ndense] element offset d*n*n of each dense slot
    mlf<N> *dense = nullptr; // [ndense][n*n]
    // position-major view of the sparse constraints for sum_k y_k A_k
    int npos = 0;
    int *pos_rc = nullptr;   // [npos] r + c*n
    int *pos_off = nullptr;  // [npos+1]
    int *pos_k = nullptr;    // contributions: global constraint index
    mlf<N> *pos_v = nullptr; //                 and value
};

// ---- elementwise ------------------------------------------------------------
template <int N>
void k_axpby(long long n, const mlf<N> &a, const mlf<N> *x, const mlf<N> &b, const mlf<N> *y, mlf<N> *out,
             cudaStream_t s);  // out = a*x + b*y (y may be null when b == 0); out may alias x or y
template <int N>
void k_copy(long long n, const mlf<N> *x, mlf<N> *out, cudaStream_t s);
template <int N>
void k_fill(long long n, mlf<N> *x, const mlf<N> &v, cudaStream_t s);  // x[i] = v
template <int N>
void k_set_identity(int n, mlf<N> *A, const mlf<N> &v, cudaStream_t s);  // A = v*I
template <int N>
void k_symmetrize(int n, mlf<N> *A, cudaStream_t s);  // Lal::getSymmetrize, sdpa_linear.cpp:457-482
template <int N>
void k_transpose(int n, const mlf<N> *A, mlf<N> *At, cudaStream_t s);
template <int N>
void k_zero_strict_upper(int n, mlf<N> *A, cudaStream_t s);

// ---- reductions (result written to a device mlf slot) -------------------------
// out[b] = sum_i x[xoff[b] + i] * y[yoff[b] + i], i < n, for b < batch (offsets in elements;
// null offset arrays mean offset 0 for every b).
template <int N>
void k_dot_batched(long long n, const mlf<N> *x, const long long *xoff, const mlf<N> *y, const long long *yoff,
                   int batch, mlf<N> *out, Workspace &ws, cudaStream_t s);
template <int N>
void k_dot(long long n, const mlf<N> *x, const mlf<N> *y, mlf<N> *out, Workspace &ws, cudaStream_t s);
template <int N>
void k_maxabs(long long n, const mlf<N> *x, mlf<N> *out, Workspace &ws, cudaStream_t s);
template <int N>
void k_trace(int n, const mlf<N> *A, mlf<N> *out, cudaStream_t s);

// ---- constraint operators (InputData::multi_InnerProductToA / multi_plusToA) ----
// g[cid] += A_cid . M  for every constraint touching the block
template <int N>
void k_constraint_inner(const BlockDev<N> &B, const mlf<N> *M, mlf<N> *g, Workspace &ws, cudaStream_t s);
// M = sum_k y_k A_k restricted to the block (overwrites M)
template <int N>
void k_constraint_plus(const BlockDev<N> &B, const mlf<N> *y, mlf<N> *M, cudaStream_t s);

// ---- Schur complement (Newton::compute_bMat_dense_SDP, sdpa_newton.cpp:1007-1096) ----
// F3 owners: B[i,j] (+ B[j,i]) += sum_{Aj} sum_{Ai} v1 v2 X[a,c] Zinv[d,b]
template <int N>
void k_schur_f3(const BlockDev<N> &B, const mlf<N> *X, const mlf<N> *Zinv, mlf<N> *bMat, int m, cudaStream_t s);
// dense copies of constraint matrices: out[t] = A_{owners[t]} (local indices)
template <int N>
void k_densify(const BlockDev<N> &B, const int *owners, int cnt, mlf<N> *out, cudaStream_t s);
// sparse partners of F1 owners: B[i,j] (+sym) += A_j . G_t for rank[j] <= rank[owner]
template <int N>
void k_schur_f1_sparse(const BlockDev<N> &B, const int *owners, int cnt, const mlf<N> *G, mlf<N> *bMat, int m,
                       cudaStream_t s);
// add a dense owner x dense-partner product table P[t + cnt*d] into B with the rank mask
template <int N>
void k_schur_f1_dense_scatter(const BlockDev<N> &B, const int *owners, int cnt, const mlf<N> *P, mlf<N> *bMat,
                              int m, cudaStream_t s);

// ---- factorisations (chol.cu) ---------------------------------------------------
// In-place lower Cholesky (Rpotrf "Lower", mplapack/Rpotrf.cpp:32-154); *info (device int)
// gets 0 or the 1-based column of the first non-positive pivot.  The strict upper
// triangle is left untouched.
template <int N>
void ml_potrf(int n, mlf<N> *A, int lda, int *info, Workspace &ws, cudaStream_t s);
// workspace ml_potrf carves beyond ws.used
template <int N>
size_t ml_potrf_workspace_bytes(int n);
// Linv = inverse of the lower-triangular L (Rtrsm on the identity, sdpa_linear.cpp:439-455);
// Linv's strict upper triangle is set to zero.
template <int N>
void ml_trtri_lower(int n, const mlf<N> *L, int ldl, mlf<N> *Linv, Workspace &ws, cudaStream_t s);
// workspace bytes ml_trtri_lower carves (beyond ws.used)
template <int N>
size_t ml_trtri_workspace_bytes(int n);
// x = (L L^T)^{-1} x (two Rtrsv, Lal::solveSystems sdpa_linear.cpp:683-695)
template <int N>
void ml_potrs(int n, const mlf<N> *L, int ldl, mlf<N> *x, Workspace &ws, cudaStream_t s);
// the same in two parts: invert the NB x NB diagonal blocks once per factor (Dinv holds
// ml_potrs_prepare_bytes), then solve any number of right-hand sides with them
template <int N>
size_t ml_potrs_prepare_bytes(int n);
template <int N>
void ml_potrs_prepare(int n, const mlf<N> *L, int ldl, mlf<N> *Dinv, cudaStream_t s);
template <int N>
void ml_potrs_solve(int n, const mlf<N> *L, int ldl, const mlf<N> *Dinv, mlf<N> *x, cudaStream_t s);
// device word inside the prepared data that a solve sets to 1 if one of its bounded
// waits timed out (the solution is then invalid); reset by every solve
template <int N>
int *ml_potrs_status(int n, mlf<N> *Dinv);

// ---- eigenvalues (eig.cu) ---------------------------------------------------------
// y = op(A) x for a dense n x n A (op: 'N' plain, 'T' transpose; A lower-triangular
// when tri != 0, entries above the diagonal ignored)
template <int N>
void k_matvec(int n, const mlf<N> *A, char op, int tri, const mlf<N> *x, mlf<N> *y, cudaStream_t s);
// r = w - alpha*q - beta*qold (alpha, beta device scalars); also writes dots:
// Smallest eigenvalue of the symmetric tridiagonal (diag d[0..k-1], offdiag e[0..k-2]) and
// the last component of its unit eigenvector (sign arbitrary): out[0] = lambda, out[1] = z_{k-1}.
template <int N>
void k_tridiag_min(int k, const mlf<N> *d, const mlf<N> *e, mlf<N> *out, int *status, cudaStream_t s,
                   const int *gate = nullptr);
// One Lanczos step k on the operator M (its columns read as rows) under device control:
// q = r / beta, w = M q, alpha = q.w -> td[k], r = w - alpha q - beta qold, beta' =
// sqrt(r.r) -> te[k], with the tridiagonal eigenvalue solve when `eig`, then the loop
// test for step k + 1 (k + 1 < n, k + 1 < kgo, beta' > 1e-16, the Ritz value or its
// error bound still moving, k + 2 < kmax).  Slots and flags in sl / ctl as described in
// eig.cu; every kernel of the step does nothing once ctl[0] is 0.  With a side stream,
// an eigenvalue step runs the tridiagonal solve there (forked after alpha, joined before
// the loop test) beside r, r.r and beta on s.
template <int N>
void k_lanczos_step(int n, const mlf<N> *M, mlf<N> *r, mlf<N> *q, mlf<N> *qold, mlf<N> *w, mlf<N> *td, mlf<N> *te,
                    mlf<N> *sl, int *ctl, int *status, int k, int eig, int kgo, int kmax, cudaStream_t s,
                    cudaStream_t side = nullptr, cudaEvent_t ev_fork = nullptr, cudaEvent_t ev_join = nullptr);
// Householder tridiagonalisation of a dense symmetric n x n (n <= 64) in place; writes
// d[0..n-1], e[0..n-2].  (Rsytrd 'L', the first stage of Rsyev.)
template <int N>
void k_tridiagonalize_small(int n, mlf<N> *A, mlf<N> *d, mlf<N> *e, cudaStream_t s);
// LP blocks (held as diagonal n x n blocks): out[0] = min_k X[k][k] L[k][k]^2, out[1] = 0.
template <int N>
void k_lp_ratio_min(int n, const mlf<N> *X, const mlf<N> *L, mlf<N> *out, cudaStream_t s);

}  // namespace sdpg
