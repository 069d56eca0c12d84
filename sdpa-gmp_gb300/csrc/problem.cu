// .dat-s / .dat and param.sdpa readers.
#include <ctype.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <sstream>

#include "ml_host.h"
#include "problem.h"

namespace sdpg {

void param_default(Param &p, int type) {
    p = Param();
    if (type == 1) {  // PARAMETER_STABLE_BUT_SLOW
        p.maxIteration = 1000;
        p.lambdaStar = 1.0e+2;
        p.betaStar = 0.2;
        p.betaBar = 0.4;
        p.gammaStar = 0.5;
        p.precision = 300;
    } else if (type == 2) {  // PARAMETER_UNSTABLE_BUT_FAST
        p.maxIteration = 100;
        p.lambdaStar = 1.0e+2;
        p.betaStar = 0.01;
        p.betaBar = 0.02;
        p.gammaStar = 0.98;
        p.precision = 100;
    }
}

bool param_read(Param &p, const char *path, std::string *err) {
    FILE *f = fopen(path, "r");
    if (!f) {
        if (err) *err = std::string("cannot open parameter file ") + path;
        return false;
    }
    // fscanf("%d%*[^\n]") / ("%lf%*[^\n]"): read the leading number of each line
    bool ok = true;
    ok &= fscanf(f, "%d%*[^\n]", &p.maxIteration) == 1;
    double *dv[] = {&p.epsilonStar, &p.lambdaStar, &p.omegaStar, &p.lowerBound, &p.upperBound,
                    &p.betaStar,    &p.betaBar,    &p.gammaStar, &p.epsilonDash};
    for (double *d : dv) ok &= fscanf(f, "%lf%*[^\n]", d) == 1;
    ok &= fscanf(f, "%d%*[^\n]", &p.precision) == 1;
    char buf[4][256];
    int nf = 0;
    for (int i = 0; i < 4; ++i)
        if (fscanf(f, "%255s %*[^\n]", buf[i]) == 1) ++nf;
    fclose(f);
    if (nf >= 1) p.xPrint = buf[0];
    if (nf >= 2) p.XPrint = buf[1];
    if (nf >= 3) p.YPrint = buf[2];
    if (nf >= 4) p.infPrint = buf[3];
    if (!ok && err) *err = std::string("malformed parameter file ") + path;
    return ok;
}

namespace {

struct Scanner {
    std::string s;
    size_t p = 0;
    // "%*[^0-9+-]": skip everything that is not a digit or sign
    bool skip() {
        while (p < s.size() && !(isdigit((unsigned char)s[p]) || s[p] == '+' || s[p] == '-')) ++p;
        return p < s.size();
    }
    bool read_int(int *v) {
        if (!skip()) return false;
        const char *b = s.c_str() + p;
        char *e = nullptr;
        long x = strtol(b, &e, 10);
        if (e == b) return false;
        p += (size_t)(e - b);
        *v = (int)x;
        return true;
    }
    bool read_num(mlf<16> *v) {
        if (!skip()) return false;
        const char *b = s.c_str() + p;
        const char *e = nullptr;
        if (!ml_parse<16>(b, v, &e) || e == b) return false;
        p += (size_t)(e - b);
        return true;
    }
};

}  // namespace

bool read_sdpa(const char *path, bool dense, RawProblem &P, std::string *err) {
    std::ifstream in(path);
    if (!in) {
        if (err) *err = std::string("cannot open data file ") + path;
        return false;
    }
    std::stringstream ss;
    std::string line;
    // title/comment lines start with '*' or '"'; the first other line holds m
    P = RawProblem();
    bool got_m = false;
    while (std::getline(in, line)) {
        if (!line.empty() && (line[0] == '*' || line[0] == '"')) {
            P.title += line + "\n";
            continue;
        }
        if (sscanf(line.c_str(), "%d", &P.m) != 1) {
            if (err) *err = "cannot read mDIM";
            return false;
        }
        got_m = true;
        break;
    }
    if (!got_m) {
        if (err) *err = "empty data file";
        return false;
    }
    ss << in.rdbuf();
    Scanner sc;
    sc.s = ss.str();
    int nBlock = 0;
    // fscanf("%d") for nBlock: skips whitespace only
    while (sc.p < sc.s.size() && isspace((unsigned char)sc.s[sc.p])) ++sc.p;
    if (!sc.read_int(&nBlock) || nBlock <= 0) {
        if (err) *err = "cannot read nBLOCK";
        return false;
    }
    P.blockStruct.resize(nBlock);
    for (int l = 0; l < nBlock; ++l)
        if (!sc.read_int(&P.blockStruct[l])) {
            if (err) *err = "cannot read bLOCKsTRUCT";
            return false;
        }
    P.c.resize(P.m);
    for (int k = 0; k < P.m; ++k)
        if (!sc.read_num(&P.c[k])) {
            if (err) *err = "cannot read the c vector";
            return false;
        }
    if (!dense) {
        while (true) {
            RawEntry e;
            int k, l, i, j;
            if (!sc.read_int(&k) || !sc.read_int(&l) || !sc.read_int(&i) || !sc.read_int(&j)) break;
            if (!sc.read_num(&e.v)) break;
            if (k < 0 || k > P.m || l < 1 || l > nBlock) {
                if (err) *err = "entry index out of range";
                return false;
            }
            const int bs = P.blockStruct[l - 1];
            const int size = bs < 0 ? -bs : bs;
            if (i < 1 || j < 1 || i > size || j > size) {
                if (err) *err = "out of range in input data";
                return false;
            }
            if (bs < 0 && i != j) {
                if (err) *err = "LP block entry off the diagonal";
                return false;
            }
            e.k = k;
            e.block = l - 1;
            e.i = i - 1;
            e.j = j - 1;
            P.entries.push_back(e);  // zero values count toward NonZeroCount as in setElement_SDP
        }
    } else {
        // dense format: F0..Fm, each block fully (SDP: size x size, LP: diagonal only)
        for (int k = 0; k <= P.m; ++k) {
            for (int l = 0; l < nBlock; ++l) {
                const int bs = P.blockStruct[l];
                if (bs >= 2) {
                    const int size = bs;
                    for (int i = 0; i < size; ++i)
                        for (int j = 0; j < size; ++j) {
                            mlf<16> v;
                            if (!sc.read_num(&v)) {
                                if (err) *err = "truncated dense data";
                                return false;
                            }
                            if (i <= j && !ml_is_zero(v)) P.entries.push_back(RawEntry{k, l, i, j, v});
                        }
                } else {
                    for (int j = 0; j < (bs < 0 ? -bs : bs); ++j) {
                        mlf<16> v;
                        if (!sc.read_num(&v)) {
                            if (err) *err = "truncated dense data";
                            return false;
                        }
                        if (!ml_is_zero(v)) P.entries.push_back(RawEntry{k, l, j, j, v});
                    }
                }
            }
        }
    }
    return true;
}

}  // namespace sdpg
