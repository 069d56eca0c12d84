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

// The reference numbers SDP blocks first (l <= number of SDP blocks, in file order) and
// addresses LP entries by one index running over all LP blocks (sdpa_io.cpp:192-217).
bool read_init(const char *path, bool sparse, int m, const std::vector<int> &blockStruct, InitPoint &ip,
               std::string *err) {
    std::ifstream in(path);
    if (!in) {
        if (err) *err = std::string("cannot open init file ") + path;
        return false;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    Scanner sc;
    sc.s = ss.str();
    auto fail = [&](const std::string &m) {
        if (err) *err = m + " in init file " + path;
        return false;
    };
    std::vector<int> sdp_blocks, lp_block, lp_local;  // file block of each SDP / LP position
    for (size_t l = 0; l < blockStruct.size(); ++l) {
        const int bs = blockStruct[l];
        if (bs >= 2) {
            sdp_blocks.push_back((int)l);
        } else {
            const int n = bs < 0 ? -bs : bs;
            for (int k = 0; k < n; ++k) {
                lp_block.push_back((int)l);
                lp_local.push_back(k);
            }
        }
    }
    ip.x0.assign(m, mlf<16>{});
    for (int k = 0; k < m; ++k)
        if (!sc.read_num(&ip.x0[k])) return fail("missing x0 entries");
    ip.entries.clear();
    if (sparse) {
        while (true) {
            int target, l, i, j;
            mlf<16> v;
            if (!sc.read_int(&target) || !sc.read_int(&l) || !sc.read_int(&i) || !sc.read_int(&j) || !sc.read_num(&v))
                break;
            if (target != 1 && target != 2) return fail("matrix selector not 1 or 2");
            if (l >= 1 && l <= (int)sdp_blocks.size()) {
                const int fb = sdp_blocks[l - 1];
                const int n = blockStruct[fb];
                if (i < 1 || j < 1 || i > n || j > n) return fail("index out of range");
                ip.entries.push_back({target, fb, i - 1, j - 1, v});
            } else if (l > (int)sdp_blocks.size()) {
                if (i != j) return fail("LP entry off the diagonal");
                if (i < 1 || i > (int)lp_block.size()) return fail("LP index out of range");
                ip.entries.push_back({target, lp_block[i - 1], lp_local[i - 1], lp_local[i - 1], v});
            } else {
                return fail("block number out of range");
            }
        }
    } else {
        // dense: Z then X, each as every SDP block in full, then all LP entries; zeros
        // and the lower triangle are skipped, as the reference skips them
        for (int target = 1; target <= 2; ++target) {
            for (int fb : sdp_blocks) {
                const int n = blockStruct[fb];
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        mlf<16> v;
                        if (!sc.read_num(&v)) return fail("missing matrix entries");
                        if (i <= j && !ml_is_zero(v)) ip.entries.push_back({target, fb, i, j, v});
                    }
            }
            for (size_t k = 0; k < lp_block.size(); ++k) {
                mlf<16> v;
                if (!sc.read_num(&v)) return fail("missing LP entries");
                if (!ml_is_zero(v)) ip.entries.push_back({target, lp_block[k], lp_local[k], lp_local[k], v});
            }
        }
    }
    return true;
}

}  // namespace sdpg
