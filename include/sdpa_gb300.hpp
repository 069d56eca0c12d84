// sdpa_gb300.hpp -- the reference's C++ class surface for the interior-point main loop,
// implemented over the C ABI of libsdpg.so (sdpg.h).
//
// SDPA-GMP reaches its hot path through C++ classes inside one binary: pinpal's main loop
// (sdpa_main.cpp:213-398) constructs Newton (sdpa_newton.h:108-168), Solutions, Residuals,
// WorkVariables (sdpa_dataset.h), StepLength, DirectionParameter, Switch,
// AverageComplementarity, RatioInitResCurrentRes, SolveInfo, Phase (sdpa_parts.h) and calls
// them in a fixed order; Lal (sdpa_linear.h:29-168) and Jal (sdpa_jordan.h:33-78) are the
// dense linear-algebra helpers underneath.  This header keeps those class names, the
// methods the main loop calls and their argument lists, so a loop written against the
// reference's classes compiles against this header and runs on the GPU.
//
// What differs from the reference, on purpose:
//   * numbers are the library's multi-limb values (sdpa::Real, exact comparisons), not
//     mpf_class; containers hold them in the library's "ml" layout (sdpg.h);
//   * the GPU solver owns the iterate.  The objects below are views of it: a value such as
//     beta.value or solveInfo.objValPrimal is refreshed from the solver by the call that
//     changes it in the reference;
//   * input comes in through IO::read(path, inputData, param, isDataSparse) (one call for
//     the reference's sequence of IO::read calls on the data file); the solver is created
//     by Newton::computeFormula_SDP (where the reference chooses the Schur formulas) with
//     the parameters given to IO::read;
//   * Solutions::initialize binds to the solver most recently created on the calling thread
//     (the reference's Solutions::initialize does not see the input either); one problem
//     per thread at a time, as the reference's process-global state implies;
//   * Chordal::ordering_bMat, Newton::initialize_bMat, WorkVariables::initialize and
//     Solutions::computeInverse have nothing left to do (the dense Schur path is the one
//     the reference takes for the supported sizes; inverses are formed by the solver);
//   * RatioInitResCurrentRes::update, AverageComplementarity::update, Residuals::update,
//     RatioInitResCurrentRes::update_exact and SolveInfo::update run as one library call
//     (sdpg_loop_after_update), made by whichever of the five comes first after
//     Solutions::update; each then refreshes its own values.
//   * Lal / Jal work on host matrices through the library's standalone GPU routines
//     (sdpg_rgemm, sdpg_rpotrf, sdpg_inv_lower, sdpg_solve_systems, sdpg_sym_min_eigen);
//     the eigenvalue helpers take blocks of at most 64 x 64.
//
// Errors: library failures throw sdpa::Error (the reference calls rError and exits);
// Newton::Mehrotra, Solutions::update and the Lal / Jal helpers return false where the
// reference returns FAILURE.
#pragma once

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sdpg.h"

namespace sdpa {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

namespace gb300 {

inline int check(int rc) {
    if (rc < 0) throw Error(rc, std::string("sdpg: ") + sdpg_last_error());
    return rc;
}

// One problem and its GPU solver, shared by the objects of one main loop.
struct Engine {
    sdpg_problem *prob = nullptr;
    sdpg_solver *solver = nullptr;
    sdpg_param param{};
    int limbs = 8;
    bool after_update_pending = false;
    bool reversed = false;
    Engine() = default;
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    ~Engine() {
        if (solver) sdpg_solver_destroy(solver);
        if (prob) sdpg_problem_free(prob);
    }
    sdpg_solver *h() const {
        if (!solver) throw Error(SDPG_ERR_STATE, "sdpa: no solver yet (Newton::computeFormula_SDP creates it)");
        return solver;
    }
};
using EnginePtr = std::shared_ptr<Engine>;

inline EnginePtr &thread_engine() {
    thread_local EnginePtr e;
    return e;
}

// copy a stdio stream's remaining contents into a temporary file (for the readers that
// take a path)
inline std::string spool(FILE *fp) {
    char name[] = "/tmp/sdpa_gb300_XXXXXX";
    const int fd = mkstemp(name);
    if (fd < 0) throw Error(SDPG_ERR_IO, "sdpa: cannot create a temporary file");
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, fp)) > 0) {
        if (write(fd, buf, n) != (ssize_t)n) {
            close(fd);
            unlink(name);
            throw Error(SDPG_ERR_IO, "sdpa: cannot write a temporary file");
        }
    }
    close(fd);
    return name;
}

}  // namespace gb300

// A multi-limb number (up to 512-bit mantissa), held with 16 limbs; comparisons are exact.
class Real {
  public:
    static constexpr int kLimbs = 16;
    Real() { set(0.0); }
    Real(double d) { set(d); }  // exact, as mpf_class x = 0.95 is
    static Real from_ml(int limbs, const void *p) {
        Real r;
        const uint32_t *w = (const uint32_t *)p;
        r.w_[0] = w[0];
        r.w_[1] = w[1];
        for (int k = 0; k < kLimbs; ++k) r.w_[2 + k] = 0;
        for (int k = 0; k < limbs; ++k) r.w_[2 + (kLimbs - limbs) + k] = w[2 + k];  // same value, wider mantissa
        return r;
    }
    double get_d() const {
        double d = 0;
        gb300::check(sdpg_ml_to_double(kLimbs, w_, 1, &d));
        return d;
    }
    std::string str(int digits = 20) const {
        char buf[512];
        gb300::check(sdpg_ml_format(kLimbs, w_, digits, buf, sizeof buf));
        return buf;
    }
    const void *ml() const { return w_; }
    friend int compare(const Real &a, const Real &b) {
        int r = 0;
        gb300::check(sdpg_ml_compare(kLimbs, a.w_, b.w_, &r));
        return r;
    }
    friend bool operator<(const Real &a, const Real &b) { return compare(a, b) < 0; }
    friend bool operator>(const Real &a, const Real &b) { return compare(a, b) > 0; }
    friend bool operator<=(const Real &a, const Real &b) { return compare(a, b) <= 0; }
    friend bool operator>=(const Real &a, const Real &b) { return compare(a, b) >= 0; }
    friend bool operator==(const Real &a, const Real &b) { return compare(a, b) == 0; }
    friend bool operator!=(const Real &a, const Real &b) { return compare(a, b) != 0; }

  private:
    void set(double d) { gb300::check(sdpg_ml_from_double(kLimbs, &d, 1, w_)); }
    uint32_t w_[2 + kLimbs];
};

// ---- containers (sdpa_struct.h:72-197), host memory in the library's ml layout --------

class Vector {
  public:
    int nDim = 0;
    int limbs = 8;
    std::vector<uint32_t> ele;  // nDim values of 2 + limbs words
    Vector() = default;
    Vector(int n, int limbs_ = 8) { initialize(n, limbs_); }
    void initialize(int n, int limbs_ = 8) {
        nDim = n;
        limbs = limbs_;
        ele.assign((size_t)n * (2 + limbs), 0u);
    }
    void *data() { return ele.data(); }
    Real get(int i) const { return Real::from_ml(limbs, &ele[(size_t)i * (2 + limbs)]); }
    void set(int i, double v) { gb300::check(sdpg_ml_from_double(limbs, &v, 1, &ele[(size_t)i * (2 + limbs)])); }
};

class DenseMatrix {
  public:
    enum Type { DENSE, COMPLETION };
    int nRow = 0, nCol = 0;
    Type type = DENSE;
    int limbs = 8;
    std::vector<uint32_t> de_ele;  // column-major, de_ele of (i, j) at i + nRow * j
    DenseMatrix() = default;
    DenseMatrix(int nr, int nc, int limbs_ = 8) { initialize(nr, nc, limbs_); }
    void initialize(int nr, int nc, int limbs_ = 8) {
        nRow = nr;
        nCol = nc;
        limbs = limbs_;
        de_ele.assign((size_t)nr * nc * (2 + limbs), 0u);
    }
    void *data() { return de_ele.data(); }
    const void *data() const { return de_ele.data(); }
    size_t bytes() const { return de_ele.size() * sizeof(uint32_t); }
    Real get(int i, int j) const { return Real::from_ml(limbs, &de_ele[((size_t)i + (size_t)nRow * j) * (2 + limbs)]); }
    void set(int i, int j, double v) {
        gb300::check(sdpg_ml_from_double(limbs, &v, 1, &de_ele[((size_t)i + (size_t)nRow * j) * (2 + limbs)]));
    }
};

class DenseLinearSpace {
  public:
    int SDP_nBlock = 0;
    std::vector<DenseMatrix> SDP_block;
    int LP_nBlock = 0;
    DenseLinearSpace() = default;
    void initialize(int SDP_nBlock_, int *SDP_blockStruct, int SOCP_nBlock, int *SOCP_blockStruct, int LP_nBlock_,
                    int limbs = 8) {
        (void)SOCP_nBlock;
        (void)SOCP_blockStruct;
        SDP_nBlock = SDP_nBlock_;
        LP_nBlock = LP_nBlock_;
        SDP_block.assign(SDP_nBlock, DenseMatrix());
        for (int l = 0; l < SDP_nBlock; ++l) SDP_block[l].initialize(SDP_blockStruct[l], SDP_blockStruct[l], limbs);
    }
    void copyFrom(DenseLinearSpace &other) { *this = other; }
};

// ---- parameters, timers, input --------------------------------------------------------

class ComputeTime {
  public:
    double Predictor = 0, Corrector = 0, StepPredictor = 0, StepCorrector = 0, xMatTime = 0, zMatTime = 0,
           invzMatTime = 0, xMatzMatTime = 0, EigxMatTime = 0, EigzMatTime = 0, EigxMatzMatTime = 0,
           makerMat = 0, makebMat = 0, B_DIAG = 0, B_F1 = 0, B_F2 = 0, B_F3 = 0, B_PRE = 0, makegVec = 0,
           choleskybMat = 0, solve = 0, sumDz = 0, makedX = 0, symmetriseDx = 0, makedXdZ = 0, updateRes = 0,
           MainLoop = 0, FileRead = 0, FileChange = 0, TotalTime = 0;
};

class Parameter {
  public:
    enum parameterType { PARAMETER_DEFAULT, PARAMETER_UNSTABLE_BUT_FAST, PARAMETER_STABLE_BUT_SLOW };
    int maxIteration = 100;
    double epsilonStar = 1e-7, lambdaStar = 1e2, omegaStar = 2.0, lowerBound = -1e5, upperBound = 1e5,
           betaStar = 0.1, betaBar = 0.2, gammaStar = 0.9, epsilonDash = 1e-7;
    int precision = 200;
    Parameter() { setDefaultParameter(); }
    void setDefaultParameter(parameterType type = PARAMETER_DEFAULT) {
        sdpg_param p;
        // sdpg_param_default: 0 default, 1 stable-but-slow, 2 unstable-but-fast
        const int t = type == PARAMETER_DEFAULT ? 0 : type == PARAMETER_STABLE_BUT_SLOW ? 1 : 2;
        gb300::check(sdpg_param_default(&p, t));
        from(p);
    }
    // Parameter::readFile (sdpa_parts.cpp:188-225): the 15-line param.sdpa layout
    void readFile(FILE *parameterFile) {
        const std::string tmp = gb300::spool(parameterFile);
        sdpg_param p = to();
        const int rc = sdpg_param_read(&p, tmp.c_str());
        unlink(tmp.c_str());
        gb300::check(rc);
        from(p);
    }
    sdpg_param to() const {
        sdpg_param p;
        p.maxIteration = maxIteration;
        p.epsilonStar = epsilonStar;
        p.lambdaStar = lambdaStar;
        p.omegaStar = omegaStar;
        p.lowerBound = lowerBound;
        p.upperBound = upperBound;
        p.betaStar = betaStar;
        p.betaBar = betaBar;
        p.gammaStar = gammaStar;
        p.epsilonDash = epsilonDash;
        p.precision = precision;
        return p;
    }
    void from(const sdpg_param &p) {
        maxIteration = p.maxIteration;
        epsilonStar = p.epsilonStar;
        lambdaStar = p.lambdaStar;
        omegaStar = p.omegaStar;
        lowerBound = p.lowerBound;
        upperBound = p.upperBound;
        betaStar = p.betaStar;
        betaBar = p.betaBar;
        gammaStar = p.gammaStar;
        epsilonDash = p.epsilonDash;
        precision = p.precision;
    }
};

class InputData {
  public:
    gb300::EnginePtr engine;
    int m = 0;
    std::vector<int> blockStruct;  // as in the data file (negative: LP block)
};

class Solutions;
class Residuals;
class WorkVariables;
class StepLength;
class DirectionParameter;
class Switch;
class AverageComplementarity;
class RatioInitResCurrentRes;
class SolveInfo;
class Phase;
class Chordal;
class Newton;

// State refreshed from the solver (sdpg_loop_values): phase, iteration and
// beta, objValPrimal, objValDual, mu, initial mu, alphaP, alphaD, thetaP, thetaD.
namespace gb300 {
struct LoopValues {
    int phase = 0, iteration = 0;
    Real v[9];
};
inline LoopValues loop_values(const EnginePtr &e) {
    LoopValues out;
    std::vector<uint32_t> buf((size_t)9 * (2 + e->limbs));
    check(sdpg_loop_values(e->h(), &out.phase, &out.iteration, buf.data()));
    for (int i = 0; i < 9; ++i) out.v[i] = Real::from_ml(e->limbs, &buf[(size_t)i * (2 + e->limbs)]);
    return out;
}
// the five bookkeeping updates after Solutions::update, once per iteration
inline void after_update(const EnginePtr &e) {
    if (e->after_update_pending) {
        e->after_update_pending = false;
        check(sdpg_loop_after_update(e->h()));
    }
}
}  // namespace gb300

class WorkVariables {
  public:
    void initialize(int m, int SDP_nBlock, int *SDP_blockStruct, int SOCP_nBlock, int *SOCP_blockStruct,
                    int LP_nBlock) {
        (void)m, (void)SDP_nBlock, (void)SDP_blockStruct, (void)SOCP_nBlock, (void)SOCP_blockStruct,
            (void)LP_nBlock;
    }
};

class Chordal {
  public:
    void ordering_bMat(int m, int nBlock, InputData &inputData, FILE *fpOut) {
        (void)m, (void)nBlock, (void)inputData, (void)fpOut;
    }
    void terminate() {}
};

class Solutions {
  public:
    int nDim = 0;
    int mDim = 0;
    DenseLinearSpace xMat, zMat;
    Vector yVec;
    gb300::EnginePtr engine;
    // Solutions::initialize (sdpa_dataset.cpp:35-60): X = Z = lambda I, y = 0 -- formed by
    // the solver at its initialisation; this binds to the calling thread's current solver.
    void initialize(int m, int SDP_nBlock, int *SDP_blockStruct, int SOCP_nBlock, int *SOCP_blockStruct,
                    int LP_nBlock, double lambda, ComputeTime &com) {
        (void)com;
        engine = gb300::thread_engine();
        if (!engine || !engine->solver)
            throw Error(SDPG_ERR_STATE, "sdpa: Solutions::initialize before Newton::computeFormula_SDP");
        engine->param.lambdaStar = lambda;
        mDim = m;
        nDim = 0;
        for (int l = 0; l < SDP_nBlock; ++l) nDim += SDP_blockStruct[l];
        nDim += LP_nBlock;
        xMat.initialize(SDP_nBlock, SDP_blockStruct, SOCP_nBlock, SOCP_blockStruct, LP_nBlock, engine->limbs);
        zMat.initialize(SDP_nBlock, SDP_blockStruct, SOCP_nBlock, SOCP_blockStruct, LP_nBlock, engine->limbs);
        yVec.initialize(m, engine->limbs);
    }
    void computeInverse(WorkVariables &work, ComputeTime &com) { (void)work, (void)com; }
    // Solutions::update (sdpa_dataset.cpp:120-143): false when the step is too short
    bool update(StepLength &alpha, Newton &newton, WorkVariables &work, ComputeTime &com);
    // copy the solver's current X, y, Z into xMat, yVec, zMat (SDP blocks)
    void fetch() {
        sdpg_solver *h = engine->h();
        for (size_t l = 0; l < xMat.SDP_block.size(); ++l) {
            gb300::check(sdpg_get_block(h, 0, (int)l, 1, xMat.SDP_block[l].data()));
            gb300::check(sdpg_get_block(h, 1, (int)l, 1, zMat.SDP_block[l].data()));
        }
        gb300::check(sdpg_get_vector(h, 0, yVec.data()));
    }
};

class Residuals {
  public:
    Real normPrimalVec, normDualMat;
    gb300::EnginePtr engine;
    Residuals() = default;
    // the initial residuals (sdpa_main.cpp:259): the solver initialises its iterate here
    Residuals(int m, int SDP_nBlock, int *SDP_blockStruct, int SOCP_nBlock, int *SOCP_blockStruct, int LP_nBlock,
              InputData &inputData, Solutions &currentPt) {
        (void)m, (void)SDP_nBlock, (void)SDP_blockStruct, (void)SOCP_nBlock, (void)SOCP_blockStruct,
            (void)LP_nBlock, (void)inputData;
        engine = currentPt.engine;
        gb300::check(sdpg_solver_initialize(engine->h()));
    }
    void copyFrom(Residuals &other) { engine = other.engine; }
    void update(int m, InputData &inputData, Solutions &currentPt, ComputeTime &com) {
        (void)m, (void)inputData, (void)com;
        engine = currentPt.engine;
        gb300::after_update(engine);
    }
    void compute(int m, InputData &inputData, Solutions &currentPt) {
        (void)m, (void)inputData;
        engine = currentPt.engine;
    }
};

class Switch {
  public:
    enum SwitchType { ON, OFF };
    SwitchType switchType;
    Switch(SwitchType t = ON) : switchType(t) {}
    void initialize(SwitchType t = ON) { switchType = t; }
    // Switch::MehrotraPredictor (sdpa_parts.cpp:605-612); the library sets the switch
    // together with DirectionParameter::MehrotraPredictor
    void MehrotraPredictor(Phase &phase);
};

class AverageComplementarity {
  public:
    Real initial, current;
    gb300::EnginePtr engine;
    AverageComplementarity(double lambdaStar = 1.0) : initial(lambdaStar * lambdaStar), current(lambdaStar * lambdaStar) {}
    void initialize(Solutions &currentPt) { engine = currentPt.engine; refresh(); }
    void update(Solutions &currentPt) {
        engine = currentPt.engine;
        gb300::after_update(engine);
        refresh();
    }
    void refresh() {
        const gb300::LoopValues v = gb300::loop_values(engine);
        current = v.v[3];
        initial = v.v[4];
    }
};

class SolveInfo {
  public:
    enum phaseType { noINFO, pFEAS, dFEAS, pdFEAS, pdINF, pFEAS_dINF, pINF_dFEAS, pdOPT, pUNBD, dUNBD };
    Real objValPrimal, objValDual;
    gb300::EnginePtr engine;
    SolveInfo() = default;
    SolveInfo(InputData &inputData, Solutions &currentPt, const Real &mu0, double omegaStar) {
        (void)inputData, (void)mu0, (void)omegaStar;
        engine = currentPt.engine;
        refresh();
    }
    void update(double lambdaStar, InputData &inputData, Solutions &currentPt, Residuals &currentRes,
                AverageComplementarity &mu, RatioInitResCurrentRes &theta, Parameter &param) {
        (void)lambdaStar, (void)inputData, (void)currentRes, (void)mu, (void)theta, (void)param;
        engine = currentPt.engine;
        gb300::after_update(engine);
        refresh();
    }
    void refresh() {
        const gb300::LoopValues v = gb300::loop_values(engine);
        objValPrimal = v.v[1];
        objValDual = v.v[2];
    }
};

class RatioInitResCurrentRes {
  public:
    Real primal, dual;
    gb300::EnginePtr engine;
    RatioInitResCurrentRes() = default;
    RatioInitResCurrentRes(Parameter &param, Residuals &initRes) {
        (void)param;
        engine = initRes.engine;
        refresh();
    }
    void update(Switch &reduction, StepLength &alpha);
    void update_exact(Residuals &initRes, Residuals &currentRes) {
        (void)initRes;
        engine = currentRes.engine;
        gb300::after_update(engine);
        refresh();
    }
    void refresh() {
        const gb300::LoopValues v = gb300::loop_values(engine);
        primal = v.v[7];
        dual = v.v[8];
    }
};

class Phase {
  public:
    SolveInfo::phaseType value = SolveInfo::noINFO;
    int nDim = 0;
    gb300::EnginePtr engine;
    Phase() = default;
    Phase(Residuals &initRes, SolveInfo &solveInfo, Parameter &param, int nDim_) : nDim(nDim_) {
        (void)solveInfo, (void)param;
        engine = initRes.engine;
        refresh();
    }
    // Phase::updateCheck (sdpa_parts.cpp:932-1011)
    bool updateCheck(Residuals &currentRes, SolveInfo &solveInfo, Parameter &param) {
        (void)solveInfo, (void)param;
        engine = currentRes.engine;
        const bool go = gb300::check(sdpg_loop_phase_check(engine->h())) == 1;
        refresh();
        return go;
    }
    // Phase::reverse (REVERSE_PRIMAL_DUAL): the primal / dual roles of the result swap
    void reverse() {
        static const SolveInfo::phaseType rev[] = {SolveInfo::noINFO,     SolveInfo::dFEAS, SolveInfo::pFEAS,
                                                   SolveInfo::pdFEAS,     SolveInfo::pdINF, SolveInfo::pINF_dFEAS,
                                                   SolveInfo::pFEAS_dINF, SolveInfo::pdOPT, SolveInfo::dUNBD,
                                                   SolveInfo::pUNBD};
        value = rev[value];
        if (engine) engine->reversed = true;
    }
    void refresh() { value = (SolveInfo::phaseType)gb300::loop_values(engine).phase; }
};

inline void Switch::MehrotraPredictor(Phase &phase) { (void)phase; }

class DirectionParameter {
  public:
    Real value;
    gb300::EnginePtr engine;
    DirectionParameter(double betaStar = 0.0) : value(betaStar) {}
    // DirectionParameter::MehrotraPredictor (sdpa_parts.cpp:543-553) with the switch of
    // Switch::MehrotraPredictor
    void MehrotraPredictor(Phase &phase, Switch &reduction, Parameter &param) {
        (void)reduction, (void)param;
        engine = phase.engine;
        gb300::check(sdpg_loop_direction(engine->h(), 0));
        refresh();
    }
    // DirectionParameter::MehrotraCorrector (sdpa_parts.cpp:555-586)
    void MehrotraCorrector(Phase &phase, StepLength &alpha, Solutions &currentPt, Newton &newton,
                           AverageComplementarity &mu, Parameter &param) {
        (void)phase, (void)alpha, (void)newton, (void)mu, (void)param;
        engine = currentPt.engine;
        gb300::check(sdpg_loop_direction(engine->h(), 1));
        refresh();
    }
    void refresh() { value = gb300::loop_values(engine).v[0]; }
};

class Newton {
  public:
    enum WHICH_DIRECTION { PREDICTOR, CORRECTOR };
    gb300::EnginePtr engine;
    Newton() = default;
    Newton(int m, int SDP_nBlock, int *SDP_blockStruct, int SOCP_nBlock, int *SOCP_blockStruct, int LP_nBlock) {
        (void)m, (void)SDP_nBlock, (void)SDP_blockStruct, (void)SOCP_nBlock, (void)SOCP_blockStruct,
            (void)LP_nBlock;
    }
    void initialize_bMat(int m, Chordal &chordal, InputData &inputData, FILE *fpOut) {
        (void)m, (void)chordal, (void)fpOut;
        engine = inputData.engine;
    }
    // Newton::computeFormula_SDP (sdpa_newton.cpp:694-819): the solver chooses F1 / F2 / F3
    // per constraint and block with the reference's cost model while it is set up, here.
    void computeFormula_SDP(InputData &inputData, double DenseRatio, double Kappa) {
        (void)DenseRatio, (void)Kappa;
        engine = inputData.engine;
        if (!engine || !engine->prob) throw Error(SDPG_ERR_STATE, "sdpa: no input data (IO::read)");
        if (!engine->solver) {
            int err = 0;
            engine->solver = sdpg_solver_create(engine->prob, &engine->param, 0, nullptr, &err);
            if (!engine->solver) gb300::check(err ? err : SDPG_ERR_CUDA);
            engine->limbs = gb300::check(sdpg_solver_limbs(engine->solver));
        }
        gb300::thread_engine() = engine;
    }
    // Newton::Mehrotra (sdpa_newton.cpp:1375-1414): false when the Schur Cholesky fails
    bool Mehrotra(WHICH_DIRECTION direction, InputData &inputData, Solutions &currentPt, Residuals &currentRes,
                  AverageComplementarity &mu, DirectionParameter &beta, Switch &reduction, Phase &phase,
                  WorkVariables &work, ComputeTime &com) {
        (void)inputData, (void)currentRes, (void)mu, (void)beta, (void)reduction, (void)phase, (void)work, (void)com;
        engine = currentPt.engine;
        const int rc = sdpg_newton(engine->h(), direction == CORRECTOR ? 1 : 0);
        if (rc == SDPG_ERR_NOT_PD) return false;
        gb300::check(rc);
        return true;
    }
};

class StepLength {
  public:
    Real primal, dual;
    gb300::EnginePtr engine;
    // StepLength::MehrotraPredictor (sdpa_parts.cpp:362-411)
    void MehrotraPredictor(InputData &inputData, Solutions &currentPt, Phase &phase, Newton &newton,
                           WorkVariables &work, ComputeTime &com) {
        (void)inputData, (void)phase, (void)newton, (void)work, (void)com;
        engine = currentPt.engine;
        gb300::check(sdpg_step_length(engine->h(), 0));
        refresh();
    }
    // StepLength::MehrotraCorrector (sdpa_parts.cpp:412-523)
    void MehrotraCorrector(InputData &inputData, Solutions &currentPt, Phase &phase, Switch &reduction,
                           Newton &newton, AverageComplementarity &mu, RatioInitResCurrentRes &theta,
                           WorkVariables &work, Parameter &param, ComputeTime &com) {
        (void)inputData, (void)phase, (void)reduction, (void)newton, (void)mu, (void)theta, (void)work,
            (void)param, (void)com;
        engine = currentPt.engine;
        gb300::check(sdpg_step_length(engine->h(), 1));
        refresh();
    }
    void refresh() {
        const gb300::LoopValues v = gb300::loop_values(engine);
        primal = v.v[5];
        dual = v.v[6];
    }
};

inline bool Solutions::update(StepLength &alpha, Newton &newton, WorkVariables &work, ComputeTime &com) {
    (void)alpha, (void)newton, (void)work, (void)com;
    const int rc = sdpg_loop_update(engine->h());
    if (rc == SDPG_ERR_NOT_PD) return false;
    gb300::check(rc);
    engine->after_update_pending = true;
    return true;
}

inline void RatioInitResCurrentRes::update(Switch &reduction, StepLength &alpha) {
    (void)reduction;
    engine = alpha.engine;
    gb300::after_update(engine);
    refresh();
}

// ---- input and output (sdpa_io.h) ------------------------------------------------------

class IO {
  public:
    // The data file (.dat-s when isDataSparse, else .dat) with the parameters the solver
    // will use: IO::read's sequence over the data file (sdpa_io.cpp:123-750) in one call.
    static void read(const char *dataPath, InputData &inputData, Parameter &param, bool isDataSparse = true) {
        int err = 0;
        auto e = std::make_shared<gb300::Engine>();
        e->prob = sdpg_problem_read(dataPath, isDataSparse ? 0 : 1, &err);
        if (!e->prob) gb300::check(err ? err : SDPG_ERR_IO);
        e->param = param.to();
        inputData.engine = e;
    }
    // The initial-point file (sdpa_io.cpp:150-276) into the solver behind currentPt: the
    // argument list of the reference's IO::read(fpInit, xMat, yVec, zMat, inputSparse),
    // with the Solutions whose containers they are.
    static void read(FILE *fpInit, Solutions &currentPt, bool inputSparse) {
        const std::string tmp = gb300::spool(fpInit);
        const int rc = sdpg_solver_read_initial_point(currentPt.engine->h(), tmp.c_str(), inputSparse ? 1 : 0);
        unlink(tmp.c_str());
        gb300::check(rc);
    }
    static void printHeader(FILE *fpout, FILE *Display) {
        const char *hdr = "   mu      thetaP  thetaD  objP      objD      alphaP  alphaD  beta \n";
        if (fpout) fputs(hdr, fpout);
        if (Display) fputs(hdr, Display);
    }
    // IO::printOneIteration (sdpa_io.cpp:764-796)
    static void printOneIteration(int pIteration, AverageComplementarity &mu, RatioInitResCurrentRes &theta,
                                  SolveInfo &solveInfo, StepLength &alpha, DirectionParameter &beta, FILE *fpout,
                                  FILE *Display) {
        (void)pIteration, (void)mu, (void)theta, (void)solveInfo, (void)beta;
        gb300::check(sdpg_loop_record(alpha.engine->h(), fpout, Display));
    }
    // IO::printLastInfo (sdpa_io.cpp:996-1184): the summary, parameters, times and the
    // solution; the final residuals (Residuals::compute) are taken here
    static void printLastInfo(int pIteration, AverageComplementarity &mu, RatioInitResCurrentRes &theta,
                              SolveInfo &solveInfo, StepLength &alpha, DirectionParameter &beta,
                              Residuals &currentRes, Phase &phase, Solutions &currentPt, double cputime,
                              InputData &inputData, WorkVariables &work, ComputeTime &com, Parameter &param,
                              FILE *fpout, FILE *Display, bool printTime = true) {
        (void)pIteration, (void)mu, (void)theta, (void)solveInfo, (void)alpha, (void)beta, (void)currentRes,
            (void)phase, (void)cputime, (void)inputData, (void)work, (void)com, (void)param, (void)printTime;
        gb300::check(sdpg_loop_finish(currentPt.engine->h(), fpout, Display));
    }
    static void printLastInfo(int pIteration, AverageComplementarity &mu, RatioInitResCurrentRes &theta,
                              SolveInfo &solveInfo, StepLength &alpha, DirectionParameter &beta,
                              Residuals &currentRes, Phase &phase, Solutions &currentPt, double cputime, int nBlock,
                              int *blockStruct, int *blockType, int *blockNumber, InputData &inputData,
                              WorkVariables &work, ComputeTime &com, Parameter &param, FILE *fpout, FILE *Display,
                              bool printTime = true) {
        (void)nBlock, (void)blockStruct, (void)blockType, (void)blockNumber;
        printLastInfo(pIteration, mu, theta, solveInfo, alpha, beta, currentRes, phase, currentPt, cputime,
                      inputData, work, com, param, fpout, Display, printTime);
    }
};

// ---- Lal / Jal: dense multi-limb linear algebra on host matrices ----------------------

class Lal {
  public:
    // Lal::multiply (sdpa_linear.cpp:856-875): retMat = scalar * aMat * bMat
    static bool multiply(DenseMatrix &retMat, DenseMatrix &aMat, DenseMatrix &bMat, Real *scalar = nullptr) {
        return gemm('N', 'N', retMat, aMat, bMat, scalar);
    }
    // retMat = scalar * aMat^T * bMat
    static bool tran_multiply(DenseMatrix &retMat, DenseMatrix &aMat, DenseMatrix &bMat, Real *scalar = nullptr) {
        return gemm('T', 'N', retMat, aMat, bMat, scalar);
    }
    // retMat = scalar * aMat * bMat^T
    static bool multiply_tran(DenseMatrix &retMat, DenseMatrix &aMat, DenseMatrix &bMat, Real *scalar = nullptr) {
        return gemm('N', 'T', retMat, aMat, bMat, scalar);
    }
    // Lal::choleskyFactorWithAdjust (sdpa_linear.cpp:608-681): in-place lower Rpotrf
    static bool choleskyFactorWithAdjust(DenseMatrix &aMat) {
        int info = 0;
        gb300::check(sdpg_rpotrf(aMat.limbs, aMat.nRow, aMat.data(), aMat.nRow, &info));
        return info == 0;
    }
    // Lal::getCholesky (sdpa_linear.cpp:342-390): retMat = lower factor of aMat, upper zero
    static bool getCholesky(DenseMatrix &retMat, DenseMatrix &aMat) {
        retMat = aMat;
        if (!choleskyFactorWithAdjust(retMat)) return false;
        const double zero = 0.0;
        for (int j = 1; j < retMat.nCol; ++j)
            for (int i = 0; i < j; ++i)
                gb300::check(sdpg_ml_from_double(retMat.limbs, &zero, 1,
                                                 &retMat.de_ele[((size_t)i + (size_t)retMat.nRow * j) *
                                                                (2 + retMat.limbs)]));
        return true;
    }
    // Lal::getInvLowTriangularMatrix (sdpa_linear.cpp:439-455)
    static bool getInvLowTriangularMatrix(DenseMatrix &retMat, DenseMatrix &aMat) {
        retMat.initialize(aMat.nRow, aMat.nCol, aMat.limbs);
        gb300::check(sdpg_inv_lower(aMat.limbs, aMat.nRow, aMat.data(), aMat.nRow, retMat.data()));
        return true;
    }
    // Lal::solveSystems (sdpa_linear.cpp:683-695): xVec = (L L^T)^-1 bVec, L = the factor in aMat
    static bool solveSystems(Vector &xVec, DenseMatrix &aMat, Vector &bVec) {
        xVec = bVec;
        gb300::check(sdpg_solve_systems(aMat.limbs, aMat.nRow, aMat.data(), aMat.nRow, xVec.data()));
        return true;
    }
    // Lal::getMinEigenValue (sdpa_linear.cpp:126-158): smallest eigenvalue (n <= 64)
    static Real getMinEigenValue(DenseMatrix &aMat, Vector &eigenVec, Vector &workVec) {
        (void)eigenVec, (void)workVec;
        std::vector<uint32_t> out(2 + aMat.limbs);
        gb300::check(sdpg_sym_min_eigen(aMat.limbs, aMat.nRow, aMat.data(), out.data()));
        return Real::from_ml(aMat.limbs, out.data());
    }

  private:
    static bool gemm(char ta, char tb, DenseMatrix &C, DenseMatrix &A, DenseMatrix &B, Real *scalar) {
        const int m = ta == 'N' ? A.nRow : A.nCol, k = ta == 'N' ? A.nCol : A.nRow;
        const int n = tb == 'N' ? B.nCol : B.nRow;
        const int limbs = A.limbs;
        C.initialize(m, n, limbs);
        std::vector<uint32_t> alpha(2 + limbs), beta(2 + limbs);
        const double one = 1.0, zero = 0.0;
        gb300::check(sdpg_ml_from_double(limbs, &one, 1, alpha.data()));
        gb300::check(sdpg_ml_from_double(limbs, &zero, 1, beta.data()));
        if (scalar) {  // narrow the 16-limb scalar to the matrices' limbs (truncation)
            const uint32_t *w = (const uint32_t *)scalar->ml();
            alpha[0] = w[0];
            alpha[1] = w[1];
            for (int q = 0; q < limbs; ++q) alpha[2 + q] = w[2 + (Real::kLimbs - limbs) + q];
        }
        gb300::check(sdpg_rgemm(limbs, ta, tb, m, n, k, alpha.data(), A.data(), A.nRow, B.data(), B.nRow,
                                beta.data(), C.data(), C.nRow));
        return true;
    }
};

class Jal {
  public:
    // Jal::multiply (sdpa_jordan.cpp:173-215), block by block
    static bool multiply(DenseLinearSpace &retMat, DenseLinearSpace &aMat, DenseLinearSpace &bMat,
                         Real *scalar = nullptr) {
        retMat.SDP_nBlock = aMat.SDP_nBlock;
        retMat.SDP_block.resize(aMat.SDP_block.size());
        for (size_t l = 0; l < aMat.SDP_block.size(); ++l)
            if (!Lal::multiply(retMat.SDP_block[l], aMat.SDP_block[l], bMat.SDP_block[l], scalar)) return false;
        return true;
    }
    // Jal::ns_jordan_triple_product (sdpa_jordan.cpp:336-340): retMat = aMat bMat cMat
    static bool ns_jordan_triple_product(DenseLinearSpace &retMat, DenseLinearSpace &aMat, DenseLinearSpace &bMat,
                                         DenseLinearSpace &cMat, DenseLinearSpace &work) {
        return multiply(work, aMat, bMat) && multiply(retMat, work, cMat);
    }
    // Jal::getInvChol (sdpa_jordan.cpp:123-139): invCholMat = L^-1 with aMat = L L^T
    static bool getInvChol(DenseLinearSpace &invCholMat, DenseLinearSpace &aMat, DenseLinearSpace &workMat) {
        workMat.SDP_block.resize(aMat.SDP_block.size());
        invCholMat.SDP_nBlock = aMat.SDP_nBlock;
        invCholMat.SDP_block.resize(aMat.SDP_block.size());
        for (size_t l = 0; l < aMat.SDP_block.size(); ++l) {
            if (!Lal::getCholesky(workMat.SDP_block[l], aMat.SDP_block[l])) return false;
            Lal::getInvLowTriangularMatrix(invCholMat.SDP_block[l], workMat.SDP_block[l]);
        }
        return true;
    }
    // Jal::getInvCholAndInv (sdpa_jordan.cpp:141-171): also inverseMat = L^-T L^-1
    static bool getInvCholAndInv(DenseLinearSpace &invCholMat, DenseLinearSpace &inverseMat, DenseLinearSpace &aMat,
                                 DenseLinearSpace &workMat) {
        if (!getInvChol(invCholMat, aMat, workMat)) return false;
        inverseMat.SDP_nBlock = aMat.SDP_nBlock;
        inverseMat.SDP_block.resize(aMat.SDP_block.size());
        for (size_t l = 0; l < aMat.SDP_block.size(); ++l)
            Lal::tran_multiply(inverseMat.SDP_block[l], invCholMat.SDP_block[l], invCholMat.SDP_block[l]);
        return true;
    }
    // Jal::getMinEigen (sdpa_jordan.cpp:55-88) on host blocks of at most 64 x 64: the
    // smallest eigenvalue over the blocks of lMat xMat lMat^T
    static Real getMinEigen(DenseLinearSpace &lMat, DenseLinearSpace &xMat, WorkVariables &work) {
        (void)work;
        Real best(1e300);
        for (size_t l = 0; l < xMat.SDP_block.size(); ++l) {
            DenseMatrix t, s;
            Lal::multiply(t, lMat.SDP_block[l], xMat.SDP_block[l]);
            Lal::multiply_tran(s, t, lMat.SDP_block[l]);
            Vector ev, wv;
            const Real v = Lal::getMinEigenValue(s, ev, wv);
            if (v < best) best = v;
        }
        return best;
    }
};

}  // namespace sdpa
