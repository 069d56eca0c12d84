// Precision-independent problem description and parameters, plus the SDPA
// .dat-s / param.sdpa readers (sdpa_io.cpp:123-141, 626-663; sdpa_parts.cpp:136-225).
#pragma once
#include <stdio.h>

#include <string>
#include <vector>

#include "ml.cuh"

namespace sdpg {

// Interior-point parameters (the reference's Parameter class).
struct Param {
    int maxIteration = 200;
    double epsilonStar = 1.0e-30;
    double lambdaStar = 1.0e+4;
    double omegaStar = 2.0;
    double lowerBound = -1.0e+5;
    double upperBound = 1.0e+5;
    double betaStar = 0.1;
    double betaBar = 0.3;
    double gammaStar = 0.9;
    double epsilonDash = 1.0e-30;
    int precision = 200;
    std::string xPrint = "%+50.40Fe", XPrint = "%+50.40Fe", YPrint = "%+50.40Fe", infPrint = "%+50.40Fe";
};

// Parameter::setDefaultParameter (sdpa_parts.cpp:136-181); type 0 default,
// 1 stable-but-slow, 2 unstable-but-fast.
void param_default(Param &p, int type = 0);
// Parameter::readFile (sdpa_parts.cpp:188-225): 11 numbers then 4 format strings.
bool param_read(Param &p, const char *path, std::string *err);

// One stored entry of F_k (k = 0 is F0; the solver's C is -F0), 0-based indices.
struct RawEntry {
    int k, block, i, j;
    mlf<16> v;
};

struct RawProblem {
    std::string title;  // comment/title lines, as read
    int m = 0;
    std::vector<int> blockStruct;  // as in the file (negative = LP block)
    std::vector<mlf<16>> c;        // the c vector (the solver's b)
    std::vector<RawEntry> entries;
};

// IO::read for the sparse format (.dat-s); dense .dat when `dense` is true.
bool read_sdpa(const char *path, bool dense, RawProblem &P, std::string *err);

// An initial point (IO::read of -id / -is files, sdpa_io.cpp:150-276): the first m
// numbers are x0 (the solver's y = -x0), then entries of the two matrices, target 1
// the solver's Z (the user's primal matrix) and target 2 its X.  Entries are kept as
// given, with blocks in the data file's numbering (0-based) and indices within the
// block; entries not given keep the lambdaStar * I start (as in the reference).
struct InitEntry {
    int target, block, i, j;
    mlf<16> v;
};
struct InitPoint {
    std::vector<mlf<16>> x0;
    std::vector<InitEntry> entries;
};
bool read_init(const char *path, bool sparse, int m, const std::vector<int> &blockStruct, InitPoint &ip,
               std::string *err);

template <int N>
inline mlf<N> narrow(const mlf<16> &x) {
    mlf<N> r;
    r.e = x.e;
    r.s = x.s;
    for (int k = 0; k < N; ++k) r.m[k] = x.m[16 - N + k];
    return r;
}

}  // namespace sdpg
