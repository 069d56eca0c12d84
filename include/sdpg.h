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
/* One value through a GMP printf format for an mpf operand, as gmp_fprintf renders the
 * result file's xPrint / XPrint / YPrint (e.g. "%+50.40Fe"; conversions e E f g G, flags
 * "-+ 0#", rounded half up like mpf_get_str).  Returns the length written. */
int sdpg_ml_format_gmp(int limbs, const void *v, const char *fmt, char *buf, int cap);
int sdpg_ml_from_double(int limbs, const double *x, long long n, void *out);
int sdpg_ml_to_double(int limbs, const void *v, long long n, double *out);
int sdpg_ml_from_mpf(int limbs, const sdpg_mpf_t *src, long long n, void *out);
/* dst[i]._mp_d must hold _mp_prec + 1 limbs (as GMP allocates). */
int sdpg_ml_to_mpf(int limbs, const void *v, long long n, sdpg_mpf_t *dst);
/* *result = -1, 0 or 1 as a < b, a == b, a > b (exact); mpf_cmp's role. */
int sdpg_ml_compare(int limbs, const void *a, const void *b, int *result);
/* Elementwise host arithmetic in the ml format (SDPG_OP_*); b is ignored for SQRT. */
int sdpg_ml_host_op(int limbs, int op, long long n, const void *a, const void *b, void *out);

/* C = alpha*op(A)*op(B) + beta*C  -- replaces Rgemm (mplapack/Rgemm_omp.cpp:41-127,
 * dispatching to Rgemm_{NN,NT,TN,TT}_omp.cpp) as called by Lal::multiply
 * (sdpa_linear.cpp:856-875).  transa/transb: 'N' or 'T'. */
int sdpg_rgemm(int limbs, char transa, char transb, int m, int n, int k, const void *alpha, const void *A,
               int lda, const void *B, int ldb, const void *beta, void *C, int ldc);
/* Scratch: the library keeps one device workspace per (calling host thread, current
 * device, stream) and grows it on demand (cudaMalloc / cudaFree, which wait for the
 * device).  Calls on one stream reuse it in stream order; calls on different streams
 * or devices, or from different threads, never share scratch. */
int sdpg_rgemm_device(int limbs, char transa, char transb, int m, int n, int k, const void *alpha,
                      const void *A, int lda, const void *B, int ldb, const void *beta, void *C, int ldc,
                      void *stream);

/* Size of the fixed device scratch behind sdpg_rgemm_device_noalloc (64 MiB). */
#define SDPG_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* The same product as sdpg_rgemm_device, for callers that must not have the library
 * allocate device memory: programs whose device memory is all held by their own pool
 * allocator, or latency-critical loops where an allocation (which synchronises the
 * device and can fail when memory is short) is not acceptable.  It has no counterpart
 * in the reference.  Its scratch is one fixed device array of SDPG_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library holds until the process exits; the call makes no
 * cudaMalloc / cudaFree and no allocating library call.  The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress), so make it before any
 * stream capture.  Products needing more scratch than the limit (about 880 x 880 x 880
 * at 256 bits) return SDPG_ERR_TOO_LARGE without launching anything.  All calls share
 * the one array: calls whose work can overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Nothing in the array needs to
 * start at zero; each call writes every scratch byte it reads. */
int sdpg_rgemm_device_noalloc(int limbs, char transa, char transb, int m, int n, int k, const void *alpha,
                              const void *A, int lda, const void *B, int ldb, const void *beta, void *C,
                              int ldc, void *stream);


/* ---- factorisations and eigenvalues (standalone, host buffers) ---------------- */

/* In-place lower Cholesky; *info = 0 or the 1-based column of the first
 * non-positive pivot -- replaces Rpotrf("Lower") (mplapack/Rpotrf.cpp:32-154) as
 * called by Lal::choleskyFactorWithAdjust (sdpa_linear.cpp:608-616).  Returns
 * SDPG_ERR_TIMEOUT (with *info = -1) if a bounded wait inside a panel gave up. */
int sdpg_rpotrf(int limbs, int n, void *A, int lda, int *info);
/* Linv (n x n, ld n) = L^{-1} for lower-triangular L -- replaces
 * Lal::getInvLowTriangularMatrix (sdpa_linear.cpp:439-455, Rtrsm on I). */
int sdpg_inv_lower(int limbs, int n, const void *L, int ldl, void *Linv);
/* x := (L L^T)^{-1} x -- replaces Lal::solveSystems (sdpa_linear.cpp:683-695, two Rtrsv). */
int sdpg_solve_systems(int limbs, int n, const void *L, int ldl, void *x);
/* Smallest eigenvalue of the symmetric tridiagonal (d[0..k-1], e[0..k-2]) and the
 * last component of its unit eigenvector (out2[0], out2[1]) -- the values
 * Lal::getMinEigen reads from Rsteqr (sdpa_linear.cpp:65-112). */
int sdpg_tridiag_min(int limbs, int k, const void *d, const void *e, void *out2);
/* Smallest eigenvalue of a dense symmetric n x n (n <= 64, lower triangle read) --
 * replaces Lal::getMinEigenValue (sdpa_linear.cpp:126-158, Rsyev 'N' 'L').
 * SDPG_ERR_NOCONV (out still written) when the Newton iteration on the characteristic
 * polynomial did not reach full precision within its step limit, as happens for a
 * tight cluster of smallest eigenvalues (a nearly singular matrix). */
int sdpg_sym_min_eigen(int limbs, int n, const void *A, void *out);

/* ---- the interior-point solver ------------------------------------------------ */

/* Parameter::{setDefaultParameter,readFile} (sdpa_parts.cpp:136-225); type 0 default,
 * 1 stable-but-slow, 2 unstable-but-fast (the -pt presets). */
typedef struct {
    int maxIteration;
    double epsilonStar, lambdaStar, omegaStar, lowerBound, upperBound, betaStar, betaBar, gammaStar,
        epsilonDash;
    int precision;
} sdpg_param;
int sdpg_param_default(sdpg_param *p, int type);
int sdpg_param_read(sdpg_param *p, const char *path);

/* Problem data in SDPA form (IO::read, sdpa_io.cpp:123-141, 410-663): F_0..F_m and c.
 * Indices are 1-based as in .dat-s; entry k = 0 is F_0 (the solver's C = -F_0). */
typedef struct sdpg_problem sdpg_problem;
sdpg_problem *sdpg_problem_new(int m, int nBlock, const int *blockStruct, int *err);
sdpg_problem *sdpg_problem_read(const char *path, int dense_format, int *err);
void sdpg_problem_free(sdpg_problem *p);
int sdpg_problem_set_c(sdpg_problem *p, int k, const char *text);
int sdpg_problem_add_entry(sdpg_problem *p, int k, int block, int i, int j, const char *text);
int sdpg_problem_add_entry_mpf(sdpg_problem *p, int k, int block, int i, int j, const sdpg_mpf_t *v);
/* Bulk input (no reference counterpart; the reference builds F_k entry by entry in
 * IO::read): c_k from a double (exact), and the upper triangle of a dense symmetric
 * n x n block of F_k from column-major doubles (each exact), n = the block size. */
int sdpg_problem_set_c_double(sdpg_problem *p, int k, double v);
int sdpg_problem_add_dense(sdpg_problem *p, int k, int block, int n, const double *A);

/* GPU-resident solver state (the reference's Solutions, Residuals, Newton and
 * WorkVariables, sdpa_dataset.h:29-177, sdpa_newton.h:33-168).  stream may be NULL. */
typedef struct sdpg_solver sdpg_solver;
sdpg_solver *sdpg_solver_create(const sdpg_problem *p, const sdpg_param *param, int device, void *stream,
                                int *err);
void sdpg_solver_destroy(sdpg_solver *h);
int sdpg_solver_limbs(sdpg_solver *h);
int sdpg_solver_dims(sdpg_solver *h, int *m, int *nblocks, int *block_sizes, int cap);
/* Solutions::initialize (sdpa_dataset.cpp:35-60) + initial Residuals, mu, theta, SolveInfo, Phase
 * (sdpa_main.cpp:229-287). */
int sdpg_solver_initialize(sdpg_solver *h);
/* The predictor-corrector loop of pinpal (sdpa_main.cpp:294-398); writes the
 * reference's iteration table and summary to out_path (may be NULL) and stdout
 * when asked; returns the iteration count. */
int sdpg_solver_run(sdpg_solver *h, const char *out_path, int print_to_stdout);
/* One pass of the main-loop body (predictor, step, corrector, step, update, residuals,
 * sdpa_main.cpp:294-384): returns 1 when an iteration was made, 0 once the loop has
 * stopped (phase decided, iteration limit, Schur Cholesky failure, or cannot move). */
int sdpg_solver_iterate(sdpg_solver *h);
/* pinpal's main loop one step at a time (sdpa_main.cpp:294-398), in its order; the C++
 * classes of sdpa_gb300.hpp (Phase, DirectionParameter, StepLength, Solutions, ...) call
 * these.  sdpg_solver_iterate is the sequence predictor-direction .. after-update.
 *   sdpg_loop_phase_check     Phase::updateCheck (sdpa_parts.cpp:932-1011): 1 go on, 0 stop
 *                             (initialises the solver on its first call)
 *   sdpg_loop_direction       corrector 0: Switch::MehrotraPredictor and
 *                             DirectionParameter::MehrotraPredictor (sdpa_parts.cpp:543-553,
 *                             605-612); 1: DirectionParameter::MehrotraCorrector (:555-586)
 *   sdpg_loop_corrector_break 1 if the phase is pdFEAS and (beta > 5 or objValPrimal <
 *                             objValDual): the loop's break before the corrector
 *                             (sdpa_main.cpp:335-339)
 *   sdpg_loop_record          IO::printOneIteration (sdpa_io.cpp:764-796) to out_file and
 *                             display_file (FILE *, either may be NULL); records the row
 *   sdpg_loop_update          Solutions::update (sdpa_dataset.cpp:120-143); SDPG_ERR_NOT_PD
 *                             when the step is too short ("cannot move")
 *   sdpg_loop_after_update    RatioInitResCurrentRes::update, AverageComplementarity::update,
 *                             Residuals::update, RatioInitResCurrentRes::update_exact,
 *                             SolveInfo::update, and the iteration count (sdpa_main.cpp:374-382)
 *   sdpg_loop_finish          Residuals::compute, Phase::reverse and IO::printLastInfo
 *                             (sdpa_main.cpp:387-398) to out_file / display_file
 *   sdpg_loop_values          the phase (as the loop sees it, not reversed), the iteration
 *                             count and 9 ml values: beta, objValPrimal (C.X), objValDual
 *                             (b.y), mu, initial mu, alphaP, alphaD, thetaP, thetaD */
int sdpg_loop_phase_check(sdpg_solver *h);
int sdpg_loop_direction(sdpg_solver *h, int corrector);
int sdpg_loop_corrector_break(sdpg_solver *h);
int sdpg_loop_record(sdpg_solver *h, void *out_file, void *display_file);
int sdpg_loop_update(sdpg_solver *h);
int sdpg_loop_after_update(sdpg_solver *h);
int sdpg_loop_finish(sdpg_solver *h, void *out_file, void *display_file);
int sdpg_loop_values(sdpg_solver *h, int *phase, int *iteration, void *out_ml9);
/* Newton::Mehrotra (sdpa_newton.cpp:1375-1414); direction 0 predictor, 1 corrector.
 * Returns SDPG_ERR_NOT_PD when the Schur Cholesky fails (the reference's FAILURE). */
int sdpg_newton(sdpg_solver *h, int direction);
/* StepLength::MehrotraPredictor / MehrotraCorrector (sdpa_parts.cpp:362-523). */
int sdpg_step_length(sdpg_solver *h, int direction);
/* Solutions::update + computeInverse (sdpa_dataset.cpp:96-143); SDPG_ERR_NOT_PD when
 * the step is too short or X / Z lost positive definiteness ("cannot move"). */
int sdpg_update(sdpg_solver *h);
/* Residuals::compute (sdpa_dataset.cpp:625-646). */
int sdpg_residuals(sdpg_solver *h);
/* Newton::Make_bMat (sdpa_newton.cpp:1251-1272) at the current iterate: m x m Schur matrix. */
int sdpg_make_schur(sdpg_solver *h, void *out_ml);
/* Newton::Make_gVec (sdpa_newton.cpp:840-895): right-hand side g (m). */
int sdpg_make_gvec(sdpg_solver *h, int direction, void *out_ml);
/* Jal::getMinEigen (sdpa_jordan.cpp:55-88) of L_X^{-1} dX L_X^{-T} (side 0) or the Z side (1). */
int sdpg_min_eigen(sdpg_solver *h, int side, void *out_ml);
/* [phase, iteration, objValPrimal, objValDual, mu, relative gap, p.feas.error,
 *  d.feas.error, alphaP, alphaD, beta, digits] as the reference prints them. */
int sdpg_solution_info(sdpg_solver *h, double *out12);
/* 0 objValPrimal, 1 objValDual, 2 mu, 3 relative gap, 4 p.feas.error, 5 d.feas.error as %e text. */
int sdpg_solution_text(sdpg_solver *h, int which, int digits, char *buf, int cap);
/* The printed xVec (= -y); form 0 doubles, 1 ml elements. */
int sdpg_get_xvec(sdpg_solver *h, int form, void *out);
/* which: 0 X, 1 Z, 2 dX, 3 dZ, 4 Z^-1, 5 L_X^-1, 6 L_Z^-1, 7 C, 8 dual residual (block 0-based). */
int sdpg_get_block(sdpg_solver *h, int which, int block, int form, void *out);
/* which: 0 y, 1 dy, 2 b, 3 primal residual p (ml elements, length m). */
int sdpg_get_vector(sdpg_solver *h, int which, void *out_ml);
/* Per-phase milliseconds: schur, cholesky, rMat+gVec, dX/dZ, step length, update, residual, total
 * (the reference's ComputeTime, sdpa_parts.cpp:26-123). */
int sdpg_solver_timers(sdpg_solver *h, double *out8);
/* Iteration table rows (9 doubles each: it, mu, thetaP, thetaD, objP, objD, alphaP, alphaD, beta). */
int sdpg_solver_history(sdpg_solver *h, double *out, int cap);
/* Multi-limb multiply-adds issued through the GEMM since the last counter reset. */
long long sdpg_solver_gemm_macs(sdpg_solver *h);
int sdpg_solver_reset_counters(sdpg_solver *h);
/* enable: 1 on, 0 off, -1 unchanged.  out3 (may be NULL): digit-GEMM kernel milliseconds,
 * launches and multi-limb MACs since the last counter reset (events on the solver's stream). */
int sdpg_solver_gemm_profile(sdpg_solver *h, int enable, double *out3);
/* Bytes copied host->device and device->host by this solver so far (setup included). */
int sdpg_solver_io_bytes(sdpg_solver *h, long long *h2d, long long *d2h);

/* ---- instrumentation (no reference counterpart) ---------------------------- */
/* Total kernel launches made by the library in this process. */
unsigned long long sdpg_launch_count(void);
/* GEMM method for 256-bit products: 0 (default) the residue-number-system path on the
 * tcgen05 tensor cores wherever it applies (K <= 16384, not tiny), 1 the integer digit
 * GEMM everywhere, 2 the residue path for every product with K <= 16384 (tests).
 * Returns the previous method.  Both paths meet the same error bound. */
int sdpg_set_gemm_method(int method);
/* *flag = non-zero if a tensor-core GEMM kernel or a standalone Cholesky (sdpg_rpotrf)
 * on `device` ever gave up a bounded wait (its results are then invalid).  The flag is
 * sticky: it is never cleared, for the life of the process.  Each solver also has its
 * own word for its GEMMs and Cholesky panels, cleared when it is created and checked
 * every iteration (a time-out there fails that solver with SDPG_ERR_TIMEOUT, not the
 * other solvers on the device). */
int sdpg_tensor_error(int device, int *flag);
/* Per-kernel timing (no reference counterpart; the reference's ComputeTime times whole
 * phases).  While enabled, every kernel the library launches outside a stream capture is
 * bracketed by a pair of CUDA events on its own stream, and the solvers run their
 * captured sequences as plain launches.  sdpg_kernel_timing returns the previous state.
 * sdpg_kernel_times waits for the recorded kernels, writes one line per kernel name,
 * "name launches milliseconds work", sorted by name, into buf, forgets the records and
 * returns the number of lines (SDPG_ERR_TOO_LARGE if cap is too small).  `work` is the
 * launches' summed algorithmic work where the library states one: for
 * tc_residue_kernel, crt_exp_kernel, tc_reconstruct_kernel and lz_matvec_kernel the
 * bytes the kernel must move (multi-limb entries read, residue planes written, ...), for
 * tc_modgemm_kernel the fp16 tensor flops 2 M N K per residue GEMM; 0 elsewhere. */
int sdpg_kernel_timing(int enable);
int sdpg_kernel_times(char *buf, int cap);
/* Test hook (no reference counterpart): the budget, in GPU clock cycles, of the
 * tensor-core GEMM kernel's primary waits (TMA data arriving, ring stages freed) and of
 * the Cholesky panel's row waits (rows give up with *info = -1 and the error word set);
 * cycles <= 0 restores the default of about one second.  With a budget shorter than a
 * copy takes, those waits give up: the kernel records the time-out in the caller's
 * error word and the sticky device flag (sdpg_tensor_error), waits with the full
 * budget for the copies and products it already issued, frees its tensor memory and
 * returns; a solver then fails with SDPG_ERR_TIMEOUT.  Returns the previous setting. */
long long sdpg_set_tensor_wait_budget(long long cycles);
/* Measured throughput of signed 32x32->64 multiply-adds (IMAD.WIDE) on one GPU, the
 * instruction the multi-limb GEMM is built from; the plain path's roofline denominator. */
int sdpg_probe_imad_wide(int device, double *ops_per_second);
/* Measured throughput of one tensor instruction on one GPU, in multiply-add operations
 * (2 per MAC) per second, from fixed operands with no memory traffic (no reference
 * counterpart: it records why the residue GEMM uses fp16 products).  kind 0:
 * tcgen05.mma kind::f16 (fp16 x fp16 -> fp32, M = 128, N = 256, one CTA per SM);
 * 1: mma.sync m16n8k32 s8 x s8 -> s32 (tcgen05.mma kind::i8 does not exist for sm_103a);
 * 2: mma.sync m16n8k16 f16 x f16 -> f32. */
int sdpg_probe_tensor_rate(int device, int kind, double *ops_per_second);
/* Batched solves (no reference counterpart; the reference solves one problem per
 * process): `count` problems with one parameter set (NULL: defaults), up to
 * `concurrency` solvers in flight at once, one host thread and its own CUDA streams
 * each, so many small latency-bound solves share the GPU.  info12[12 i] and
 * iterations[i] (either may be NULL) receive each problem's summary and iteration
 * count, or iterations[i] < 0 (an SDPG_ERR_* code) if that solve failed.  Returns the
 * number of problems solved without error. */
int sdpg_solve_batch(int count, sdpg_problem *const *problems, const sdpg_param *param, int device, int concurrency,
                     double *info12, int *iterations);
/* Read data + param, solve, write the result file: `sdpa_gmp -ds data -o out -p param`
 * (main / pinpal, sdpa_main.cpp:43-461, 501-677).  Returns iterations; info12 as above. */
int sdpg_solve_file(const char *data_path, const char *param_path, const char *out_path, int device,
                    double *info12);
/* The same with, if print_to_stdout, the iteration table and summary also on stdout:
 * what the command-line driver sdpa_gmp_gb300 calls.  param (may be NULL) gives the
 * parameters directly and param_path is then only echoed in the header; with param NULL
 * a param_path is read as a param.sdpa file, and without either the defaults apply.
 * data_dense: the data file is in the dense .dat format (-dd) instead of .dat-s (-ds).
 * init_path (may be NULL): an initial-point file, sparse (-is) or dense (-id) format. */
int sdpg_solve_file_ex(const char *data_path, int data_dense, const sdpg_param *param, const char *param_path,
                       const char *init_path, int init_sparse, const char *out_path, int device, int print_to_stdout,
                       double *info12);

/* ---- learned parameter proposal (no reference counterpart) ------------------
 * A fully connected FP32 network (6 inputs, three hidden layers of 64 tanh units,
 * 2 outputs) run and trained by the library's own CUDA kernels.  Inputs per sample:
 *   log10 mu, log10 max-norm primal residual, log10 max-norm dual residual,
 *   previous primal step length, previous dual step length,
 *   the corrector centering value of the reference's rule (DirectionParameter::
 *   MehrotraCorrector, sdpa_parts.cpp:555-586) at this iteration;
 * outputs: log10 lambdaStar (used at the initial point, Solutions::initialize,
 * sdpa_dataset.cpp:35-60) and the corrector's beta.  Parameters are a flat float array
 * (W1[64][6] b1 W2[64][64] b2 W3[64][64] b3 W4[2][64] b4, row-major [out][in]); the
 * scaling block holds x_mean[6] x_std[6] y_mean[2] y_std[2]: the network sees
 * (x - x_mean) / x_std and its output z is reported as y_mean + y_std z. */
#define SDPG_POLICY_INPUTS 6
#define SDPG_POLICY_OUTPUTS 2
#define SDPG_POLICY_PARAMS 8898
#define SDPG_POLICY_SCALE 16
typedef struct sdpg_policy sdpg_policy;
/* Glorot-uniform weights from a fixed seed, zero biases, identity scaling. */
int sdpg_policy_create(int device, sdpg_policy **out);
void sdpg_policy_destroy(sdpg_policy *p);
/* Either pointer may be NULL (left unchanged); resets the optimiser state. */
int sdpg_policy_set(sdpg_policy *p, const float *params, const float *scale);
int sdpg_policy_get(sdpg_policy *p, float *params, float *scale);
/* y[count][2] = network(x[count][6]) (host buffers). */
int sdpg_policy_forward(sdpg_policy *p, const float *x, int count, float *y);
/* Loss sum_i,o mask[i][o] (z[i][o] - (t[i][o] - y_mean[o]) / y_std[o])^2 / count in
 * standardised units, and its gradient with respect to every parameter. */
int sdpg_policy_gradient(sdpg_policy *p, const float *x, const float *t, const float *mask, int count, float *grad,
                         float *loss);
/* Adam (lr, 0.9, 0.999, 1e-8) on that loss over shuffled mini-batches of `batch`
 * samples for `epochs` passes; epoch_loss[e] (may be NULL) = mean batch loss of pass e. */
int sdpg_policy_train(sdpg_policy *p, const float *x, const float *t, const float *mask, int count, int epochs,
                      int batch, float lr, unsigned long long seed, float *epoch_loss);
/* IO::read of an initial-point file (sdpa_io.cpp:150-276; sparse: the -is format,
 * otherwise -id): x0 then the user's primal matrix (target 1) and dual matrix (target 2).
 * The next initialize() starts from it (main, sdpa_main.cpp:237-277): entries not given
 * keep lambdaStar * I, y = -x0, mu0 = X.Z / n.  SDPG_ERR_NOT_PD from initialize() if a
 * matrix is not positive definite. */
int sdpg_solver_read_initial_point(sdpg_solver *h, const char *path, int sparse);
/* Attach (NULL detaches) a policy to a solver on the same device.  flags: 1 propose the
 * corrector beta each iteration, 2 propose lambdaStar at initialize().  A proposed beta
 * whose step fails the checks (the predicted mu must fall by a factor 1 - min(alphaP,
 * alphaD) / 4 or more; a residual that is not yet zero needs a step length of at least
 * 0.5) is replaced by the reference's own value for that iteration.  The policy must outlive its use and not be trained meanwhile. */
int sdpg_solver_set_policy(sdpg_solver *h, sdpg_policy *p, int flags);
/* [proposals, fallbacks, lambdaStar in use, lambdaStar proposed (0 if none)]. */
int sdpg_solver_policy_stats(sdpg_solver *h, double *out4);
/* Per-iteration policy inputs recorded by the solver (with or without a policy): up to
 * cap rows of 6 floats, one per row of sdpg_solver_history.  Returns the row count. */
int sdpg_solver_features(sdpg_solver *h, float *out, int cap);

#ifdef __cplusplus
}
#endif
#endif /* SDPG_H */
