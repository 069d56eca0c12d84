// A driver written against include/sdpa_gb300.hpp only, in the shape of SDPA-GMP's
// pinpal main loop (sdpa_main.cpp:213-398): the same classes, constructed and called in
// the same order, with the GPU library underneath.
//
//   pinpal_loop DATA.dat-s PARAM [OUT] [INIT.ini-s]
//
// Prints the iteration table and summary to stdout (and to OUT when given).
#include <stdio.h>

#include <algorithm>

#include "sdpa_gb300.hpp"

using namespace sdpa;

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: pinpal_loop DATA PARAM [OUT] [INIT]\n");
        return 2;
    }
    try {
        Parameter param;
        param.setDefaultParameter(Parameter::PARAMETER_DEFAULT);
        FILE *fpParameter = fopen(argv[2], "r");
        if (!fpParameter) {
            fprintf(stderr, "cannot open %s\n", argv[2]);
            return 2;
        }
        param.readFile(fpParameter);
        fclose(fpParameter);
        FILE *fpOut = argc > 3 ? fopen(argv[3], "w") : nullptr;
        FILE *Display = stdout;

        InputData inputData;
        IO::read(argv[1], inputData, param, true);
        ComputeTime com;
        const double KAPPA = 1.2;  // the reference's cost-model constant (sdpa_main.cpp:27)

        int m = 0, nBlocks = 0;
        // the block structure comes from the solver once it exists; the constructors below
        // only need it for their own containers
        Newton newton;
        Chordal chordal;
        newton.initialize_bMat(m, chordal, inputData, fpOut);
        newton.computeFormula_SDP(inputData, 0.0, KAPPA);
        chordal.terminate();

        int sizes[4096];
        gb300::check(sdpg_solver_dims(inputData.engine->h(), &m, &nBlocks, sizes, 4096));
        std::vector<int> sdpStruct(sizes, sizes + nBlocks);
        const int SDP_nBlock = nBlocks, SOCP_nBlock = 0, LP_nBlock = 0;

        Solutions currentPt;
        WorkVariables work;
        currentPt.initialize(m, SDP_nBlock, sdpStruct.data(), SOCP_nBlock, nullptr, LP_nBlock, param.lambdaStar, com);
        work.initialize(m, SDP_nBlock, sdpStruct.data(), SOCP_nBlock, nullptr, LP_nBlock);
        const bool isInitFile = argc > 4;
        if (isInitFile) {
            FILE *fpInit = fopen(argv[4], "r");
            if (!fpInit) {
                fprintf(stderr, "cannot open %s\n", argv[4]);
                return 2;
            }
            IO::read(fpInit, currentPt, true);
            fclose(fpInit);
            currentPt.computeInverse(work, com);
        }

        Residuals initRes(m, SDP_nBlock, sdpStruct.data(), SOCP_nBlock, nullptr, LP_nBlock, inputData, currentPt);
        Residuals currentRes;
        currentRes.copyFrom(initRes);

        StepLength alpha;
        DirectionParameter beta(param.betaStar);
        Switch reduction(Switch::ON);
        AverageComplementarity mu(param.lambdaStar);
        if (isInitFile) mu.initialize(currentPt);
        RatioInitResCurrentRes theta(param, initRes);
        SolveInfo solveInfo(inputData, currentPt, mu.initial, param.omegaStar);
        Phase phase(initRes, solveInfo, param, currentPt.nDim);

        int pIteration = 0;
        IO::printHeader(fpOut, Display);
        while (phase.updateCheck(currentRes, solveInfo, param) && pIteration < param.maxIteration) {
            // predictor
            reduction.MehrotraPredictor(phase);
            beta.MehrotraPredictor(phase, reduction, param);
            if (!newton.Mehrotra(Newton::PREDICTOR, inputData, currentPt, currentRes, mu, beta, reduction, phase, work,
                                 com))
                break;
            alpha.MehrotraPredictor(inputData, currentPt, phase, newton, work, com);
            // corrector
            beta.MehrotraCorrector(phase, alpha, currentPt, newton, mu, param);
            if (phase.value == SolveInfo::pdFEAS &&
                (beta.value > 5 || solveInfo.objValPrimal < solveInfo.objValDual))
                break;
            newton.Mehrotra(Newton::CORRECTOR, inputData, currentPt, currentRes, mu, beta, reduction, phase, work,
                            com);
            alpha.MehrotraCorrector(inputData, currentPt, phase, reduction, newton, mu, theta, work, param, com);
            IO::printOneIteration(pIteration, mu, theta, solveInfo, alpha, beta, fpOut, Display);
            if (!currentPt.update(alpha, newton, work, com)) break;  // cannot move
            theta.update(reduction, alpha);
            mu.update(currentPt);
            currentRes.update(m, inputData, currentPt, com);
            theta.update_exact(initRes, currentRes);
            solveInfo.update(param.lambdaStar, inputData, currentPt, currentRes, mu, theta, param);
            ++pIteration;
        }
        currentRes.compute(m, inputData, currentPt);
        phase.reverse();
        IO::printLastInfo(pIteration, mu, theta, solveInfo, alpha, beta, currentRes, phase, currentPt, 0.0, inputData,
                          work, com, param, fpOut, Display);
        if (fpOut) fclose(fpOut);
        // a host-side check of the Lal helpers on the final iterate: X is singular at the
        // optimum, so S = X X^T + diag(1, 2, .., n) (via Lal::multiply_tran) has every
        // eigenvalue >= 1, a simple smallest one, and a Cholesky factor
        // (Lal::choleskyFactorWithAdjust)
        currentPt.fetch();
        for (auto &blk : currentPt.xMat.SDP_block) {
            if (blk.nRow > 64) continue;
            DenseMatrix S;
            Lal::multiply_tran(S, blk, blk);
            for (int i = 0; i < S.nRow; ++i) {
                const double one = 1.0 + i;
                std::vector<uint32_t> a(2 + S.limbs), b(2 + S.limbs);
                uint32_t *sii = &S.de_ele[((size_t)i + (size_t)S.nRow * i) * (2 + S.limbs)];
                gb300::check(sdpg_ml_from_double(S.limbs, &one, 1, b.data()));
                gb300::check(sdpg_ml_host_op(S.limbs, SDPG_OP_ADD, 1, sii, b.data(), a.data()));
                std::copy(a.begin(), a.end(), sii);
            }
            Vector ev, wv;
            const Real lmin = Lal::getMinEigenValue(S, ev, wv);
            DenseMatrix F = S;
            const bool chol = Lal::choleskyFactorWithAdjust(F);
            printf("lal: block %d min eigenvalue of X X^T + D %s, Cholesky %s\n", blk.nRow, lmin.str(6).c_str(),
                   chol ? "ok" : "failed");
            if (!(lmin >= 0.999) || !chol) {
                fprintf(stderr, "the Lal check on the final iterate failed\n");
                return 1;
            }
        }
        printf("pinpal_loop: %d iterations, phase value %d\n", pIteration, (int)phase.value);
    } catch (const Error &e) {
        fprintf(stderr, "pinpal_loop: %s (code %d)\n", e.what(), e.code);
        return 1;
    }
    return 0;
}
