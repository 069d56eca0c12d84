// The GPU-resident interior-point state and the Newton step (SDPA-GMP's
// Newton / Jal / Lal hot path with its Solutions, Residuals and IPM control).
#pragma once
#include <stdio.h>

#include <array>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "mlp.cuh"
#include "problem.h"
#include "real.h"

namespace sdpg {

// Phase values (SolveInfo::phaseType, sdpa_parts.h).
enum Phase {
    noINFO = 0,
    pFEAS,
    dFEAS,
    pdFEAS,
    pdINF,
    pFEAS_dINF,
    pINF_dFEAS,
    pdOPT,
    pUNBD,
    dUNBD
};
const char *phase_name(int phase);

// Per-phase wall-clock accounting (ComputeTime, sdpa_parts.h:46-83), milliseconds.
struct Timers {
    double schur = 0, cholesky = 0, rmat_gvec = 0, dxdz = 0, steplen = 0, update = 0, residual = 0, total = 0;
};

struct IterRecord {
    int it;
    double mu, thetaP, thetaD, objP, objD, alphaP, alphaD, beta;
};

// Type-erased solver interface used by the C ABI.
class SolverBase {
  public:
    virtual ~SolverBase() {}
    virtual int limbs() const = 0;
    virtual void initialize() = 0;                          // Solutions::initialize + residuals
    virtual int run(FILE *out, FILE *display) = 0;          // pinpal main loop; returns iterations
    // One pass of the main-loop body (sdpa_main.cpp:294-384): 1 = iterated, 0 = the loop
    // condition or a break stopped it (phase decided, Cholesky failure, cannot move).
    virtual int iterate(FILE *out) = 0;
    // The main loop's steps one at a time, in the order pinpal calls them
    // (sdpa_main.cpp:294-398); run() / iterate() are these steps in sequence.
    virtual bool loop_phase_check() = 0;                    // Phase::updateCheck
    virtual void loop_direction(int corrector) = 0;         // Switch + DirectionParameter::Mehrotra*
    virtual bool loop_corrector_break() const = 0;          // the pdFEAS stopping rule (:337)
    virtual void loop_record(FILE *out, FILE *display) = 0;  // IO::printOneIteration
    virtual bool loop_update() = 0;                          // Solutions::update ("cannot move")
    virtual void loop_after_update() = 0;  // theta, mu, Residuals::update, SolveInfo::update, iteration
    virtual void loop_finish(FILE *out, FILE *display) = 0;  // Residuals::compute, Phase::reverse, printLastInfo
    // the loop's state as the reference's objects hold it: the phase (not reversed), the
    // iteration count, and 9 ml values: beta, objValPrimal (C.X), objValDual (b.y), mu,
    // initial mu, alphaP, alphaD, thetaP, thetaD
    virtual void loop_values(int *phase, int *iteration, void *out9) const = 0;
    virtual bool newton(int corrector) = 0;                 // Newton::Mehrotra
    virtual void step_length(int corrector) = 0;            // StepLength::Mehrotra{Predictor,Corrector}
    virtual bool update() = 0;                              // Solutions::update
    virtual void residuals() = 0;                           // Residuals::compute
    virtual int phase() const = 0;
    virtual int iteration() const = 0;
    virtual void info(double *out12) const = 0;             // see sdpg_solution_info
    virtual std::string info_text(int which, int digits) const = 0;
    virtual void get_y(void *out, int form) const = 0;      // form 0: double, 1: ml
    // which: 0 X, 1 Z, 2 dX, 3 dZ, 4 Z^-1, 5 L_X^-1, 6 L_Z^-1, 7 C, 8 dual residual
    virtual void get_block(int which, int block, void *out, int form) const = 0;
    virtual void make_bmat(void *out_ml) = 0;               // Newton::Make_bMat at the current iterate
    virtual void make_gvec(int corrector, void *out_ml) = 0;  // Newton::Make_gVec
    virtual void min_eigen(int side, void *out_ml) = 0;     // Jal::getMinEigen(L_X^-1,dX) / (L_Z^-1,dZ)
    virtual void get_vec(int which, void *out_ml) const = 0;  // 0 y, 1 dy, 2 b, 3 primal residual p
    virtual const Timers &timers() const = 0;
    virtual const std::vector<IterRecord> &history() const = 0;
    virtual void set_trace(FILE *f) = 0;
    virtual int m() const = 0;
    virtual int nblocks() const = 0;
    virtual int block_size(int l) const = 0;
    virtual long long gemm_macs() const = 0;                // multi-limb MACs issued through the GEMM
    virtual void reset_counters() = 0;
    // GEMM-kernel profiling: when on, every digit-GEMM launch is bracketed by CUDA events;
    // out: [kernel milliseconds, launches, multi-limb MACs] since the last reset.
    virtual void set_gemm_profiling(bool on) = 0;
    virtual void gemm_profile(double *out3) = 0;
    // bytes copied host->device and device->host since construction (setup included)
    virtual void io_bytes(long long *h2d, long long *d2h) const = 0;
    virtual void sync() = 0;
    // the data file's block structure (negative: LP block)
    virtual std::vector<int> block_structure() const = 0;
    // start from this point instead of lambdaStar * I (the -id / -is files)
    virtual void set_initial_point(const InitPoint &ip) = 0;
    // the result file after the summary block: parameters, time table, xVec / xMat / yMat
    virtual void print_result_tail(FILE *f, double file_read_seconds) = 0;
    // learned proposal (flags: 1 corrector beta, 2 lambdaStar); null detaches
    virtual void set_policy(const Policy *p, int flags) = 0;
    // [proposals, fallbacks, lambdaStar in use, lambdaStar proposed or 0]
    virtual void policy_stats(double *out4) const = 0;
    // policy inputs: row 0 at the initial point, row k + 1 at iteration k
    virtual const std::vector<std::array<float, kPolIn>> &features() const = 0;
};

// Build a solver for the SDP blocks of P at the precision in `param`.
SolverBase *make_solver(const RawProblem &P, const Param &param, int device, cudaStream_t stream);

}  // namespace sdpg
