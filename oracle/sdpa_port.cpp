// CPU restatement of the reference solver's dense-SDP interior-point method on
// GMP mpf arithmetic.
//
// TEST INFRASTRUCTURE ONLY (the "port" oracle): it is the timed CPU baseline
// on machines without the reference sources, and a second checker of the GPU
// solver.  It is never linked into, or called by, the product library.
//
// It follows the reference routine by routine (file:line cited at each) at the
// reference's default precision semantics (mpf_set_default_prec(precision),
// sdpa_parts.cpp:198-200), with the reference's only thread-parallel kernel,
// the NN matrix product (mplapack/Rgemm_NN_omp.cpp:36-74), parallelised the
// same way (OpenMP over columns).  Published algorithms stand in for the
// MPLAPACK routines the reference vendors: an unblocked right-looking Cholesky
// (Rpotrf), column substitution (Rtrsm/Rtrsv), implicit QL with shifts on the
// tridiagonal (Rsteqr/Rsterf), Householder reduction (Rsytrd).
//
// Usage: sdpa_port -ds data.dat-s -p param.sdpa [-o out] [-maxit K] [-times]
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "gmp_abi.h"

namespace {

struct F {
    mpf_t v;
    F() { mpf_init(v); }
    F(double d) {
        mpf_init(v);
        mpf_set_d(v, d);
    }
    F(const F &o) {
        mpf_init(v);
        mpf_set(v, o.v);
    }
    F &operator=(const F &o) {
        if (this != &o) mpf_set(v, o.v);
        return *this;
    }
    ~F() { mpf_clear(v); }
    double d() const { return mpf_get_d(v); }
};
F operator+(const F &a, const F &b) {
    F r;
    mpf_add(r.v, a.v, b.v);
    return r;
}
F operator-(const F &a, const F &b) {
    F r;
    mpf_sub(r.v, a.v, b.v);
    return r;
}
F operator*(const F &a, const F &b) {
    F r;
    mpf_mul(r.v, a.v, b.v);
    return r;
}
F operator/(const F &a, const F &b) {
    F r;
    mpf_div(r.v, a.v, b.v);
    return r;
}
F operator-(const F &a) {
    F r;
    mpf_neg(r.v, a.v);
    return r;
}
bool operator<(const F &a, const F &b) { return mpf_cmp(a.v, b.v) < 0; }
bool operator>(const F &a, const F &b) { return mpf_cmp(a.v, b.v) > 0; }
bool operator<=(const F &a, const F &b) { return mpf_cmp(a.v, b.v) <= 0; }
bool operator>=(const F &a, const F &b) { return mpf_cmp(a.v, b.v) >= 0; }
bool operator==(const F &a, const F &b) { return mpf_cmp(a.v, b.v) == 0; }
bool operator!=(const F &a, const F &b) { return mpf_cmp(a.v, b.v) != 0; }
F fabsF(const F &a) {
    F r;
    mpf_abs(r.v, a.v);
    return r;
}
F sqrtF(const F &a) {
    F r;
    mpf_sqrt(r.v, a.v);
    return r;
}
F fmax2(const F &a, const F &b) { return a < b ? b : a; }
F fmin2(const F &a, const F &b) { return b < a ? b : a; }
F fromInt(long i) {
    F r;
    mpf_set_si(r.v, i);
    return r;
}

struct Mat {
    int n = 0;
    std::vector<F> a;
    void init(int n_) {
        n = n_;
        a.assign((size_t)n * n, F());
    }
    F &operator()(int i, int j) { return a[i + (size_t)n * j]; }
    const F &operator()(int i, int j) const { return a[i + (size_t)n * j]; }
    void zero() {
        for (auto &x : a) mpf_set_ui(x.v, 0);
    }
    void identity(const F &s) {
        zero();
        for (int i = 0; i < n; ++i) (*this)(i, i) = s;
    }
};

// C = alpha*A*B + beta*C, the reference's Rgemm_NN_omp loop (OpenMP over columns)
void gemm_nn(Mat &C, const Mat &A, const Mat &B, const F &alpha, const F &beta) {
    const int n = C.n;
    const bool bzero = mpf_sgn(beta.v) == 0;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        mpf_t temp, templ;
        mpf_init(temp);
        mpf_init(templ);
        for (int i = 0; i < n; ++i) {
            if (bzero) mpf_set_ui(C(i, j).v, 0);
            else mpf_mul(C(i, j).v, C(i, j).v, beta.v);
        }
        for (int l = 0; l < n; ++l) {
            mpf_mul(temp, alpha.v, B(l, j).v);
            for (int i = 0; i < n; ++i) {
                mpf_mul(templ, temp, A(i, l).v);
                mpf_add(C(i, j).v, C(i, j).v, templ);
            }
        }
        mpf_clear(temp);
        mpf_clear(templ);
    }
}

// C = A*B^T (Lal::let(..,'T',..) path for the small-block eigenvalue, serial in the reference)
void gemm_nt(Mat &C, const Mat &A, const Mat &B) {
    const int n = C.n;
    mpf_t t;
    mpf_init(t);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            mpf_set_ui(C(i, j).v, 0);
            for (int l = 0; l < n; ++l) {
                mpf_mul(t, A(i, l).v, B(j, l).v);
                mpf_add(C(i, j).v, C(i, j).v, t);
            }
        }
    mpf_clear(t);
}

// inner product A.B of dense matrices (Rdot over n*n, sdpa_linear.cpp:188-202)
F dot(const std::vector<F> &a, const std::vector<F> &b) {
    F r(0.0);
    mpf_t t;
    mpf_init(t);
    for (size_t i = 0; i < a.size(); ++i) {
        mpf_mul(t, a[i].v, b[i].v);
        mpf_add(r.v, r.v, t);
    }
    mpf_clear(t);
    return r;
}

// Rpotrf("Lower") restated as unblocked right-looking Cholesky; false if not PD
bool cholesky(Mat &A) {
    const int n = A.n;
    mpf_t t;
    mpf_init(t);
    for (int j = 0; j < n; ++j) {
        if (mpf_sgn(A(j, j).v) <= 0) {
            mpf_clear(t);
            return false;
        }
        mpf_sqrt(A(j, j).v, A(j, j).v);
        for (int i = j + 1; i < n; ++i) mpf_div(A(i, j).v, A(i, j).v, A(j, j).v);
        for (int k = j + 1; k < n; ++k)
            for (int i = k; i < n; ++i) {
                mpf_mul(t, A(i, j).v, A(k, j).v);
                mpf_sub(A(i, k).v, A(i, k).v, t);
            }
    }
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < j; ++i) mpf_set_ui(A(i, j).v, 0);
    mpf_clear(t);
    return true;
}

// X = L^{-1} by forward substitution on the identity (Rtrsm, sdpa_linear.cpp:439-455)
void inv_lower(Mat &X, const Mat &L) {
    const int n = L.n;
    X.identity(F(1.0));
    mpf_t t;
    mpf_init(t);
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            if (mpf_sgn(X(i, c).v) != 0) mpf_div(X(i, c).v, X(i, c).v, L(i, i).v);
            for (int k = i + 1; k < n; ++k) {
                mpf_mul(t, L(k, i).v, X(i, c).v);
                mpf_sub(X(k, c).v, X(k, c).v, t);
            }
        }
    mpf_clear(t);
}

// Inv = L^T L (Rtrmm "Left","Lower","Transpose", sdpa_jordan.cpp:160-161)
void ltl(Mat &Inv, const Mat &L) {
    const int n = L.n;
    mpf_t t;
    mpf_init(t);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            mpf_set_ui(Inv(i, j).v, 0);
            for (int k = std::max(i, j); k < n; ++k) {
                mpf_mul(t, L(k, i).v, L(k, j).v);
                mpf_add(Inv(i, j).v, Inv(i, j).v, t);
            }
        }
    mpf_clear(t);
}

// x = (L L^T)^{-1} x (two Rtrsv, Lal::solveSystems sdpa_linear.cpp:683-695)
void potrs(const Mat &L, std::vector<F> &x) {
    const int n = L.n;
    mpf_t t;
    mpf_init(t);
    for (int j = 0; j < n; ++j) {
        mpf_div(x[j].v, x[j].v, L(j, j).v);
        for (int i = j + 1; i < n; ++i) {
            mpf_mul(t, L(i, j).v, x[j].v);
            mpf_sub(x[i].v, x[i].v, t);
        }
    }
    for (int j = n - 1; j >= 0; --j) {
        for (int i = j + 1; i < n; ++i) {
            mpf_mul(t, L(i, j).v, x[i].v);
            mpf_sub(x[j].v, x[j].v, t);
        }
        mpf_div(x[j].v, x[j].v, L(j, j).v);
    }
    mpf_clear(t);
}

F pythag(const F &a, const F &b) { return sqrtF(a * a + b * b); }

// Implicit QL with Wilkinson-type shifts on a symmetric tridiagonal (d[0..n-1],
// e[i] couples i and i+1), the published tql2/tqli algorithm that Rsteqr/Rsterf
// implement; with z != null the eigenvectors are accumulated (z = identity on entry).
bool tql(int n, std::vector<F> &d, std::vector<F> &e, std::vector<F> *z, const F &eps) {
    e.resize(n + 1, F(0.0));
    e[n - 1] = F(0.0);
    for (int l = 0; l < n; ++l) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; ++m) {
                const F dd = fabsF(d[m]) + fabsF(d[m + 1]);
                if (fabsF(e[m]) <= eps * dd) break;
            }
            if (m != l) {
                if (iter++ == 100) return false;
                F g = (d[l + 1] - d[l]) / (F(2.0) * e[l]);
                F r = pythag(g, F(1.0));
                g = d[m] - d[l] + e[l] / (g + (mpf_sgn(g.v) >= 0 ? fabsF(r) : -fabsF(r)));
                F s(1.0), c(1.0), p(0.0);
                int i;
                bool underflow = false;
                for (i = m - 1; i >= l; --i) {
                    F f = s * e[i], b = c * e[i];
                    r = pythag(f, g);
                    e[i + 1] = r;
                    if (mpf_sgn(r.v) == 0) {
                        d[i + 1] = d[i + 1] - p;
                        e[m] = F(0.0);
                        underflow = true;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + F(2.0) * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    if (z) {
                        std::vector<F> &Z = *z;
                        for (int k = 0; k < n; ++k) {
                            f = Z[k + (size_t)n * (i + 1)];
                            Z[k + (size_t)n * (i + 1)] = s * Z[k + (size_t)n * i] + c * f;
                            Z[k + (size_t)n * i] = c * Z[k + (size_t)n * i] - s * f;
                        }
                    }
                }
                if (underflow && i >= l) continue;
                d[l] = d[l] - p;
                e[l] = g;
                e[m] = F(0.0);
            }
        } while (m != l);
    }
    return true;
}

struct Entry {
    int i, j;
    F v;
};

struct Con {
    int cid = 0;
    bool dense = false;
    int nze = 0, rank = 0, formula = 0;
    std::vector<Entry> sp;  // stored entries (upper triangle as read)
    Mat D;
};

struct Blk {
    int n = 0;
    Mat C, X, Z, Zinv, LX, LZ, Dx, Dz, Rm, XRDZ, W1, W2, Dres, F;
    std::vector<Con> cons;
};

// getInnerProduct(Sparse, Dense), sdpa_linear.cpp:204-340
F sparse_dot(const Con &a, const Mat &M) {
    if (a.dense) return dot(a.D.a, M.a);
    F r(0.0), t;
    for (const Entry &e : a.sp) {
        if (e.i == e.j) t = e.v * M(e.i, e.j);
        else t = e.v * (M(e.i, e.j) + M(e.j, e.i));
        r = r + t;
    }
    return r;
}

struct Param {
    int maxIteration = 200;
    double epsilonStar = 1e-30, lambdaStar = 1e4, omegaStar = 2.0, lowerBound = -1e5, upperBound = 1e5,
           betaStar = 0.1, betaBar = 0.3, gammaStar = 0.9, epsilonDash = 1e-30;
    int precision = 200;
};

enum { noINFO = 0, pFEAS, dFEAS, pdFEAS, pdINF, pFEAS_dINF, pINF_dFEAS, pdOPT, pUNBD, dUNBD };
const char *phase_names[] = {"noINFO    ", "pFEAS     ", "dFEAS     ", "pdFEAS    ", "pdINF     ",
                             "pFEAS_dINF", "pINF_dFEAS", "pdOPT     ", "pUNBD     ", "dUNBD     "};

struct Solver {
    Param par;
    int m = 0, nDim = 0;
    std::vector<Blk> blk;
    std::vector<F> b, y, Dy, g, p;
    Mat B;
    F muInit, muCur, thP, thD, aP, aD, betaV, rho, etaP, etaD, objP, objD, normP, normD, initNormP, initNormD;
    int phase = noINFO, reductionOn = 1, iter = 0;
    F eps;

    // ---- setup (IO::read, InputData, computeFormula_SDP) ----
    bool load(const char *path) {
        std::ifstream in(path);
        if (!in) return false;
        std::string line;
        while (std::getline(in, line)) {
            if (!line.empty() && (line[0] == '*' || line[0] == '"')) continue;
            if (sscanf(line.c_str(), "%d", &m) != 1) return false;
            break;
        }
        std::stringstream ss;
        ss << in.rdbuf();
        std::string s = ss.str();
        size_t pos = 0;
        auto skip = [&]() {
            while (pos < s.size() && !(isdigit((unsigned char)s[pos]) || s[pos] == '+' || s[pos] == '-')) ++pos;
            return pos < s.size();
        };
        auto rint = [&](int *v) {
            if (!skip()) return false;
            char *e;
            long x = strtol(s.c_str() + pos, &e, 10);
            if (e == s.c_str() + pos) return false;
            pos = e - s.c_str();
            *v = (int)x;
            return true;
        };
        auto rnum = [&](F *v) {
            if (!skip()) return false;
            size_t q = pos;
            while (q < s.size() && (isdigit((unsigned char)s[q]) || strchr("+-.eE", s[q]))) ++q;
            std::string tok = s.substr(pos, q - pos);
            pos = q;
            return mpf_set_str(v->v, tok.c_str(), 10) == 0;
        };
        while (pos < s.size() && isspace((unsigned char)s[pos])) ++pos;
        int nb;
        if (!rint(&nb)) return false;
        std::vector<int> bs(nb);
        for (int l = 0; l < nb; ++l) {
            if (!rint(&bs[l])) return false;
            if (bs[l] < 2) {
                fprintf(stderr, "sdpa_port: only SDP blocks are supported\n");
                return false;
            }
        }
        b.assign(m, F());
        for (int k = 0; k < m; ++k)
            if (!rnum(&b[k])) return false;
        blk.resize(nb);
        for (int l = 0; l < nb; ++l) {
            Blk &B_ = blk[l];
            B_.n = bs[l];
            Mat *mats[] = {&B_.C, &B_.X, &B_.Z, &B_.Zinv, &B_.LX, &B_.LZ, &B_.Dx, &B_.Dz, &B_.Rm, &B_.XRDZ, &B_.W1, &B_.W2, &B_.Dres, &B_.F};
            for (Mat *M : mats) M->init(bs[l]);
        }
        std::vector<std::vector<std::vector<Entry>>> ent(m + 1, std::vector<std::vector<Entry>>(nb));
        while (true) {
            int k, l, i, j;
            F v;
            if (!rint(&k) || !rint(&l) || !rint(&i) || !rint(&j) || !rnum(&v)) break;
            ent[k][l - 1].push_back(Entry{i - 1, j - 1, v});
        }
        for (int l = 0; l < nb; ++l) {
            Blk &B_ = blk[l];
            const int n = B_.n;
            for (const Entry &e : ent[0][l]) {  // C = -F0
                B_.C(e.i, e.j) = B_.C(e.i, e.j) - e.v;
                if (e.i != e.j) B_.C(e.j, e.i) = B_.C(e.j, e.i) - e.v;
            }
            for (int k = 1; k <= m; ++k) {
                if (ent[k][l].empty()) continue;
                Con c;
                c.cid = k - 1;
                const int cnt = (int)ent[k][l].size();
                c.dense = !((double)cnt < (double)(n * n) * 0.20);  // changeToDense, sdpa_struct.cpp:491
                if (c.dense) {
                    c.D.init(n);
                    for (const Entry &e : ent[k][l]) {
                        c.D(e.i, e.j) = e.v;
                        c.D(e.j, e.i) = e.v;
                    }
                    c.nze = n * n;
                } else {
                    c.sp = ent[k][l];
                    for (const Entry &e : c.sp) c.nze += (e.i == e.j) ? 1 : 2;
                }
                B_.cons.push_back(std::move(c));
            }
            // computeFormula_SDP, sdpa_newton.cpp:694-819
            const F K(1.2);
            auto &cs = B_.cons;
            for (auto &ci : cs) {
                long up = ci.nze;
                for (auto &cj : cs) {
                    if (cj.nze < ci.nze) up += cj.nze;
                    else if (cj.nze == ci.nze && cj.cid < ci.cid) up += cj.nze;
                }
                const F nR = fromInt(n), inz = fromInt(ci.nze), upR = fromInt(up);
                const F f1 = K * nR * inz + nR * nR * nR + K * upR;
                const F f2 = K * nR * inz + K * (nR + F(1.0)) * upR;
                const F f3 = K * (F(2.0) * K * inz + F(1.0)) * upR / K;
                if (ci.dense) ci.formula = (f1 < f2) ? 0 : 1;
                else if (f1 < f2 && f1 < f3) ci.formula = 0;
                else if (f2 < f3) ci.formula = 1;
                else ci.formula = 2;
            }
        }
        nDim = 0;
        for (auto &B_ : blk) nDim += B_.n;
        y.assign(m, F(0.0));
        Dy.assign(m, F(0.0));
        g.assign(m, F(0.0));
        p.assign(m, F(0.0));
        B.init(m);
        return true;
    }

    // ---- constraint operators ----
    void multi_inner(Mat Blk::*M, std::vector<F> &out) {
        for (auto &x : out) mpf_set_ui(x.v, 0);
        for (auto &B_ : blk)
            for (auto &c : B_.cons) out[c.cid] = out[c.cid] + sparse_dot(c, B_.*M);
    }
    void multi_plus(const std::vector<F> &yy, Mat Blk::*M) {
        for (auto &B_ : blk) {
            Mat &R = B_.*M;
            R.zero();
            for (auto &c : B_.cons) {
                const F &s = yy[c.cid];
                if (c.dense) {
                    for (size_t q = 0; q < R.a.size(); ++q) R.a[q] = R.a[q] + c.D.a[q] * s;
                } else {
                    for (const Entry &e : c.sp) {
                        R(e.i, e.j) = R(e.i, e.j) + e.v * s;
                        if (e.i != e.j) R(e.j, e.i) = R(e.j, e.i) + e.v * s;
                    }
                }
            }
        }
    }
    void axpy(Mat Blk::*out, const F &a, Mat Blk::*x, const F &bb, Mat Blk::*yy) {
        for (auto &B_ : blk) {
            Mat &O = B_.*out;
            const Mat &X = B_.*x;
            for (size_t q = 0; q < O.a.size(); ++q) {
                F t = a * X.a[q];
                if (yy) t = t + bb * (B_.*yy).a[q];
                O.a[q] = t;
            }
        }
    }
    F ip(Mat Blk::*a, Mat Blk::*bb) {
        F r(0.0);
        for (auto &B_ : blk) r = r + dot((B_.*a).a, (B_.*bb).a);
        return r;
    }
    F ipv(const std::vector<F> &a, const std::vector<F> &bb) { return dot(a, bb); }

    // ---- Newton (sdpa_newton.cpp:821-1414) ----
    void compute_rMat(bool corr) {
        const F target = betaV * muCur;
        axpy(&Blk::Rm, target, &Blk::Zinv, F(0.0), nullptr);
        axpy(&Blk::Rm, F(1.0), &Blk::Rm, F(-1.0), &Blk::X);
        if (corr) {
            for (auto &B_ : blk) {
                gemm_nn(B_.W2, B_.Dx, B_.Dz, F(1.0), F(0.0));
                gemm_nn(B_.W1, B_.W2, B_.Zinv, F(1.0), F(0.0));
            }
            axpy(&Blk::Rm, F(1.0), &Blk::Rm, F(-1.0), &Blk::W1);
        }
    }
    void Make_gVec(bool corr) {
        compute_rMat(corr);
        if (phase == pFEAS || phase == noINFO) {
            if (!corr)
                for (auto &B_ : blk) {
                    gemm_nn(B_.W2, B_.X, B_.Dres, F(1.0), F(0.0));
                    gemm_nn(B_.XRDZ, B_.W2, B_.Zinv, F(1.0), F(0.0));
                }
            axpy(&Blk::W1, F(1.0), &Blk::Rm, F(-1.0), &Blk::XRDZ);
        } else {
            for (auto &B_ : blk) B_.W1.a = B_.Rm.a;
        }
        multi_inner(&Blk::W1, g);
        for (int k = 0; k < m; ++k) g[k] = p[k] - g[k];
    }
    void Make_bMat() {
        B.zero();
        for (auto &B_ : blk) {
            const int n = B_.n;
            auto &cs = B_.cons;
            for (auto &ci : cs) {
                Mat work2;
                if (ci.formula != 2) {  // F1 (F2 evaluated with the same mathematics)
                    Mat work1;
                    work1.init(n);
                    if (ci.dense) {
                        gemm_nn(work1, ci.D, B_.Zinv, F(1.0), F(0.0));
                    } else {
                        for (const Entry &e : ci.sp)
                            for (int c = 0; c < n; ++c) {
                                work1(e.i, c) = work1(e.i, c) + e.v * B_.Zinv(e.j, c);
                                if (e.i != e.j) work1(e.j, c) = work1(e.j, c) + e.v * B_.Zinv(e.i, c);
                            }
                    }
                    work2.init(n);
                    gemm_nn(work2, B_.X, work1, F(1.0), F(0.0));
                }
                for (auto &cj : cs) {
                    if (ci.nze < cj.nze || (ci.nze == cj.nze && ci.cid < cj.cid)) continue;
                    F value(0.0);
                    if (ci.formula != 2) {
                        value = sparse_dot(cj, work2);
                    } else {  // calF3, sdpa_newton.cpp:939-1005
                        for (const Entry &a1 : cj.sp) {
                            F sum(0.0);
                            for (const Entry &a2 : ci.sp) {
                                sum = sum + a2.v * B_.Zinv(a2.j, a1.j) * B_.X(a1.i, a2.i);
                                if (a2.i != a2.j) sum = sum + a2.v * B_.Zinv(a2.i, a1.j) * B_.X(a1.i, a2.j);
                            }
                            value = value + a1.v * sum;
                            if (a1.i == a1.j) continue;
                            sum = F(0.0);
                            for (const Entry &a2 : ci.sp) {
                                sum = sum + a2.v * B_.Zinv(a2.j, a1.i) * B_.X(a1.j, a2.i);
                                if (a2.i != a2.j) sum = sum + a2.v * B_.Zinv(a2.i, a1.i) * B_.X(a1.j, a2.j);
                            }
                            value = value + a1.v * sum;
                        }
                    }
                    if (ci.cid != cj.cid) {
                        B(ci.cid, cj.cid) = B(ci.cid, cj.cid) + value;
                        B(cj.cid, ci.cid) = B(cj.cid, ci.cid) + value;
                    } else {
                        B(ci.cid, ci.cid) = B(ci.cid, ci.cid) + value;
                    }
                }
            }
        }
    }
    bool newton(bool corr) {
        Make_gVec(corr);
        if (!corr) {
            Make_bMat();
            if (!cholesky(B)) return false;
        }
        Dy = g;
        potrs(B, Dy);
        multi_plus(Dy, &Blk::Dz);
        if (phase == pFEAS || phase == noINFO) axpy(&Blk::Dz, F(-1.0), &Blk::Dz, F(1.0), &Blk::Dres);
        else axpy(&Blk::Dz, F(-1.0), &Blk::Dz, F(0.0), nullptr);
        for (auto &B_ : blk) {
            gemm_nn(B_.W2, B_.X, B_.Dz, F(1.0), F(0.0));
            gemm_nn(B_.W1, B_.W2, B_.Zinv, F(1.0), F(0.0));
        }
        axpy(&Blk::Dx, F(1.0), &Blk::Rm, F(-1.0), &Blk::W1);
        for (auto &B_ : blk)  // getSymmetrize
            for (int i = 0; i < B_.n; ++i)
                for (int j = i + 1; j < B_.n; ++j) {
                    F v = (B_.Dx(i, j) + B_.Dx(j, i)) * F(0.5);
                    B_.Dx(i, j) = v;
                    B_.Dx(j, i) = v;
                }
        return true;
    }

    // ---- eigenvalues (Lal::getMinEigen / getMinEigenValue, sdpa_linear.cpp:27-158) ----
    F lanczos(const Mat &L, const Mat &X) {
        const int n = L.n;
        F min(1.0e+51), min_old(1.0e+52), error(1.0e+10);
        std::vector<F> diag(n + 1, F(1.0e50)), off(n + 1, F(0.0)), q(n, F(0.0)), qold(n), r(n, F(1.0)), w(n), tmp(n);
        F beta = sqrtF(fromInt(n));
        const F sqn = sqrtF(fromInt(n)), sqn9 = sqrtF(fromInt(n) + F(9.0));
        int k = 0, kk = 0;
        while (k < n && fromInt(k) < sqn + F(10.0) && beta > F(1.0e-16) &&
               (fabsF(min - min_old) > F(1.0e-5) * fabsF(min) + F(1.0e-8) ||
                fabsF(error * beta) > F(1.0e-2) * fabsF(min) + F(1.0e-4))) {
            qold = q;
            const F value = F(1.0) / beta;
            for (int i = 0; i < n; ++i) q[i] = r[i] * value;
            for (int j = 0; j < n; ++j) {  // w = L^T q
                F s(0.0);
                for (int i = j; i < n; ++i) s = s + L(i, j) * q[i];
                w[j] = s;
            }
            for (int i = 0; i < n; ++i) {  // tmp = X w
                F s(0.0);
                for (int j = 0; j < n; ++j) s = s + X(i, j) * w[j];
                tmp[i] = s;
            }
            for (int i = 0; i < n; ++i) {  // w = L tmp
                F s(0.0);
                for (int j = 0; j <= i; ++j) s = s + L(i, j) * tmp[j];
                w[i] = s;
            }
            const F alpha = dot(q, w);
            diag[k] = alpha;
            for (int i = 0; i < n; ++i) r[i] = w[i] - q[i] * alpha - qold[i] * beta;
            if (fromInt(kk) >= sqrtF(fromInt(k)) || k == n - 1 || fromInt(k) > sqn9) {
                kk = 0;
                const int kp1 = k + 1;
                std::vector<F> d(diag.begin(), diag.begin() + kp1), e(off.begin(), off.begin() + kp1);
                std::vector<F> Z((size_t)kp1 * kp1, F(0.0));
                for (int i = 0; i < kp1; ++i) Z[i + (size_t)kp1 * i] = F(1.0);
                if (!tql(kp1, d, e, &Z, eps)) break;
                int jmin = 0;
                for (int j = 1; j < kp1; ++j)
                    if (d[j] < d[jmin]) jmin = j;
                min_old = min;
                min = d[jmin];
                error = Z[k + (size_t)kp1 * jmin];
            }
            beta = sqrtF(dot(r, r));
            off[k] = beta;
            ++k;
            ++kk;
        }
        return min - fabsF(error * beta);
    }
    F small_min(Blk &B_, const Mat &L, const Mat &X) {
        const int n = B_.n;
        gemm_nt(B_.W2, X, L);
        gemm_nn(B_.W1, L, B_.W2, F(1.0), F(0.0));
        Mat &A = B_.W1;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) A(i, j) = A(j, i);
        std::vector<F> d(n), e(n, F(0.0));
        for (int j = 0; j + 2 < n; ++j) {  // Householder (Rsytrd)
            const int Ln = n - j - 1;
            F x0 = A(j + 1, j), sigma(0.0);
            for (int i = 1; i < Ln; ++i) sigma = sigma + A(j + 1 + i, j) * A(j + 1 + i, j);
            if (mpf_sgn(sigma.v) == 0) {
                e[j] = x0;
            } else {
                const F mu = sqrtF(x0 * x0 + sigma);
                const F bet = mpf_sgn(x0.v) >= 0 ? -mu : mu;
                const F v0 = x0 - bet, tau = (bet - x0) / bet;
                std::vector<F> v(Ln), pp(Ln), ww(Ln);
                v[0] = F(1.0);
                for (int i = 1; i < Ln; ++i) v[i] = A(j + 1 + i, j) / v0;
                for (int i = 0; i < Ln; ++i) {
                    F s(0.0);
                    for (int c = 0; c < Ln; ++c) s = s + A(j + 1 + i, j + 1 + c) * v[c];
                    pp[i] = tau * s;
                }
                F Kc(0.0);
                for (int i = 0; i < Ln; ++i) Kc = Kc + v[i] * pp[i];
                Kc = tau * Kc * F(0.5);
                for (int i = 0; i < Ln; ++i) ww[i] = pp[i] - Kc * v[i];
                for (int r2 = 0; r2 < Ln; ++r2)
                    for (int c = 0; c < Ln; ++c)
                        A(j + 1 + r2, j + 1 + c) = A(j + 1 + r2, j + 1 + c) - (v[r2] * ww[c] + ww[r2] * v[c]);
                e[j] = bet;
            }
            d[j] = A(j, j);
        }
        if (n >= 2) {
            d[n - 2] = A(n - 2, n - 2);
            e[n - 2] = A(n - 1, n - 2);
        }
        d[n - 1] = A(n - 1, n - 1);
        tql(n, d, e, nullptr, eps);
        F mn = d[0];
        for (int i = 1; i < n; ++i)
            if (d[i] < mn) mn = d[i];
        return mn;
    }
    F getMinEigen(Mat Blk::*L, Mat Blk::*X) {
        F mn(1.0e50);
        for (auto &B_ : blk) {
            const F v = B_.n > 20 ? lanczos(B_.*L, B_.*X) : small_min(B_, B_.*L, B_.*X);
            if (v < mn) mn = v;
        }
        return mn;
    }

    // ---- step length / direction parameter (sdpa_parts.cpp:298-586) ----
    void step_length(bool corr) {
        if (!corr) {
            aP = aD = F(0.9);
        } else {
            const F alphaBD(100.0);
            const F minX = getMinEigen(&Blk::LX, &Blk::Dx);
            aP = (-minX > F(1.0) / alphaBD) ? -F(1.0) / minX : alphaBD;
            const F minZ = getMinEigen(&Blk::LZ, &Blk::Dz);
            aD = (-minZ > F(1.0) / alphaBD) ? -F(1.0) / minZ : alphaBD;
            aP = F(par.gammaStar) * aP;
            aD = F(par.gammaStar) * aD;
        }
        if (phase == noINFO || phase == dFEAS) {
            if (aP > F(1.0)) aP = F(1.0);
        } else {
            if (ip(&Blk::C, &Blk::Dx) > F(0.0)) {
                if (aP > aD) aP = aD;
                if (aP > F(1.0)) aP = F(1.0);
            }
        }
        if (phase == noINFO || phase == pFEAS) {
            if (aD > F(1.0)) aD = F(1.0);
        } else {
            if (ipv(b, Dy) < F(0.0)) {
                if (aD > aP) aD = aP;
                if (aD > F(1.0)) aD = F(1.0);
            }
        }
        if (!corr) return;
        if (reductionOn && (phase == noINFO || phase == pFEAS || phase == dFEAS)) {
            const F xv = ip(&Blk::X, &Blk::Dz), uz = ip(&Blk::Dx, &Blk::Z), uv = ip(&Blk::Dx, &Blk::Dz);
            F thetaMax = fmax2((F(1.0) - aP) * thP, (F(1.0) - aD) * thD);
            F muNew = muCur + (aP * uz + aD * xv + aP * aD * uv) / fromInt(nDim);
            while (thetaMax * thetaMax * muInit > F(3.0) * muNew) {
                const F alphaMax = F(0.95) * fmax2(aP, aD);
                aP = fmin2(aP, alphaMax);
                aD = fmin2(aD, alphaMax);
                thetaMax = fmax2((F(1.0) - aP) * thP, (F(1.0) - aD) * thD);
                muNew = muCur + (aP * uz + aD * xv + aP * aD * uv) / fromInt(nDim);
                if (aP < F(1.0e-6) && aD < F(1.0e-6)) break;
            }
        }
        if (phase == pdFEAS) {
            const F oD = ipv(b, y), oP = ip(&Blk::C, &Blk::X);
            const F iD = ipv(b, Dy) * aD, iP = ip(&Blk::C, &Blk::Dx) * aP;
            const F maxRatio = (oD - oP) / (iP - iD);
            if (maxRatio > F(0.0) && maxRatio < F(1.0)) {
                aP = aP * maxRatio;
                aD = aD * maxRatio;
            }
        }
    }

    // ---- iterate update, residuals, control ----
    bool inv_chol(Blk &B_, Mat &A, Mat &Linv, Mat *Inv) {
        B_.F.a = A.a;
        if (!cholesky(B_.F)) return false;
        inv_lower(Linv, B_.F);
        if (Inv) ltl(*Inv, Linv);
        return true;
    }
    bool update() {
        axpy(&Blk::X, F(1.0), &Blk::X, aP, &Blk::Dx);
        for (int k = 0; k < m; ++k) y[k] = y[k] + Dy[k] * aD;
        axpy(&Blk::Z, F(1.0), &Blk::Z, aD, &Blk::Dz);
        if (aP < F(1.0e-4) && aD < F(1.0e-4)) return false;
        bool ok = true;
        for (auto &B_ : blk)
            if (!inv_chol(B_, B_.X, B_.LX, nullptr)) ok = false;
        for (auto &B_ : blk)
            if (!inv_chol(B_, B_.Z, B_.LZ, &B_.Zinv)) ok = false;
        return ok;
    }
    void residuals() {
        multi_inner(&Blk::X, p);
        for (int k = 0; k < m; ++k) p[k] = b[k] - p[k];
        multi_plus(y, &Blk::Dres);
        for (auto &B_ : blk)
            for (size_t q = 0; q < B_.Dres.a.size(); ++q) B_.Dres.a[q] = B_.C.a[q] - B_.Dres.a[q] - B_.Z.a[q];
        normP = F(0.0);
        for (auto &x : p)
            if (fabsF(x) > normP) normP = fabsF(x);
        normD = F(0.0);
        for (auto &B_ : blk)
            for (auto &x : B_.Dres.a)
                if (fabsF(x) > normD) normD = fabsF(x);
    }
    bool phase_check() {
        const F acc(par.epsilonDash), NONZERO(1.0e-6);
        phase = noINFO;
        if (normP <= acc) phase = (normD <= acc) ? pdFEAS : pFEAS;
        if (phase == noINFO && normD <= acc) phase = dFEAS;
        if (phase == pdFEAS) {
            const F mean = (fabsF(objP) + fabsF(objD)) / F(2.0), gap = fabsF(objP - objD);
            const F dom = mean < F(1.0) ? F(1.0) : mean;
            if (gap / dom <= F(par.epsilonStar)) {
                phase = pdOPT;
                return false;
            }
        }
        if (phase == noINFO && rho > F(1.0) + NONZERO) {
            phase = pdINF;
            return false;
        }
        if (phase == pFEAS) {
            if (objP <= -F(par.upperBound)) {
                phase = pUNBD;
                return false;
            }
            if (rho > F(1.0) + NONZERO) {
                phase = pFEAS_dINF;
                return false;
            }
        }
        if (phase == dFEAS) {
            if (objD >= -F(par.lowerBound)) {
                phase = dUNBD;
                return false;
            }
            if (rho > F(1.0) + NONZERO) {
                phase = pINF_dFEAS;
                return false;
            }
        }
        return true;
    }
    void solveInfo_update() {
        objP = ip(&Blk::C, &Blk::X);
        objD = ipv(b, y);
        const F pr = thP, du = thD, om(par.omegaStar), lam(par.lambdaStar);
        rho = F(0.0);
        const F x0z0 = fromInt(nDim) * muInit, xz = fromInt(nDim) * muCur;
        F x0z(0.0), xz0(0.0);
        for (auto &B_ : blk)
            for (int i = 0; i < B_.n; ++i) {
                x0z = x0z + lam * B_.Z(i, i);
                xz0 = xz0 + lam * B_.X(i, i);
            }
        const F acc(par.epsilonDash);
        if (normP <= acc && xz0 < etaP) etaP = xz0;
        if (normD <= acc && x0z < etaD) etaD = x0z;
        if (normP > acc && normD <= acc) rho = pr * x0z / ((pr + (F(1.0) - pr) * om) * etaD + xz);
        if (normP <= acc && normD > acc) rho = du * xz0 / ((du + (F(1.0) - du) * om) * etaP + xz);
        if (normP > acc && normD > acc)
            rho = (du * xz0 + pr * x0z) / ((pr * du + om * (pr * (F(1.0) - du) + (F(1.0) - pr) * du)) * x0z0 + xz);
    }
    void initialize() {
        const F lam(par.lambdaStar);
        const F invsq = F(1.0) / sqrtF(lam), inv = F(1.0) / lam;
        for (auto &B_ : blk) {
            B_.X.identity(lam);
            B_.Z.identity(lam);
            B_.LX.identity(invsq);
            B_.LZ.identity(invsq);
            B_.Zinv.identity(inv);
        }
        residuals();
        initNormP = normP;
        initNormD = normD;
        aP = aD = F(0.0);
        betaV = F(par.betaStar);
        reductionOn = 1;
        muInit = lam * lam;
        muCur = muInit;
        const F acc(par.epsilonDash);
        thP = initNormP < acc ? F(0.0) : F(1.0);
        thD = initNormD < acc ? F(0.0) : F(1.0);
        rho = F(1.0);
        etaP = F(par.omegaStar) * fromInt(nDim) * muInit;
        etaD = etaP;
        objP = ip(&Blk::C, &Blk::X);
        objD = ipv(b, y);
        phase_check();
        iter = 0;
    }
    std::string fmt(const char *f, const F &v) {
        char buf[256];
        gmp_snprintf(buf, sizeof buf, f, v.v);
        return buf;
    }
    void print_iter(FILE *f) {
        if (!f) return;
        fprintf(f, "%2d %s %s %s %s %s %s %s %s\n", iter, fmt("%4.1Fe", muCur).c_str(), fmt("%4.1Fe", thD).c_str(),
                fmt("%4.1Fe", thP).c_str(), fmt("%+7.2Fe", -objD).c_str(), fmt("%+7.2Fe", -objP).c_str(),
                fmt("%4.1Fe", aD).c_str(), fmt("%4.1Fe", aP).c_str(), fmt("%4.2Fe", betaV).c_str());
        fflush(f);
    }
    // one pass of the main-loop body, sdpa_main.cpp:294-384; false once stopped
    bool iterate(FILE *out) {
        if (!(phase_check() && iter < par.maxIteration)) return false;
        reductionOn = (phase == noINFO || phase == pFEAS || phase == dFEAS) ? 1 : 0;
        if (phase == pdFEAS) betaV = F(0.0);
        else betaV = reductionOn ? F(par.betaBar) : F(2.0);
        if (!newton(false)) return false;
        step_length(false);
        {
            const F xv = ip(&Blk::X, &Blk::Dz), uz = ip(&Blk::Dx, &Blk::Z), uv = ip(&Blk::Dx, &Blk::Dz);
            const F muT = muCur + (aP * uz + aD * xv + aP * aD * uv) / fromInt(nDim);
            betaV = muT / muCur;
            if (betaV < F(1.0)) betaV = betaV * betaV;
            if (phase == pdFEAS) {
                if (betaV < F(par.betaStar)) betaV = F(par.betaStar);
                if (betaV > F(1.0)) betaV = F(1.0);
            } else if (betaV < F(par.betaBar)) {
                betaV = F(par.betaBar);
            }
        }
        if (phase == pdFEAS && (betaV > F(5.0) || objP < objD)) return false;
        newton(true);
        step_length(true);
        print_iter(out);
        if (!update()) return false;
        if (reductionOn) {
            thP = fabsF((F(1.0) - aP) * thP);
            thD = fabsF((F(1.0) - aD) * thD);
        }
        muCur = ip(&Blk::X, &Blk::Z) / fromInt(nDim);
        residuals();
        thP = initNormP > F(1.0e-10) ? normP / initNormP : F(0.0);
        thD = initNormD > F(1.0e-10) ? normD / initNormD : F(0.0);
        solveInfo_update();
        ++iter;
        return true;
    }
};

bool read_param(Param &p, const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return false;
    bool ok = fscanf(f, "%d%*[^\n]", &p.maxIteration) == 1;
    double *dv[] = {&p.epsilonStar, &p.lambdaStar, &p.omegaStar, &p.lowerBound, &p.upperBound,
                    &p.betaStar,    &p.betaBar,    &p.gammaStar, &p.epsilonDash};
    for (double *d : dv) ok &= fscanf(f, "%lf%*[^\n]", d) == 1;
    ok &= fscanf(f, "%d%*[^\n]", &p.precision) == 1;
    fclose(f);
    return ok;
}

}  // namespace

int main(int argc, char **argv) {
    const char *data = nullptr, *param = nullptr, *outp = nullptr;
    int maxit = -1;
    bool times = false;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-ds") && i + 1 < argc) data = argv[++i];
        else if (!strcmp(argv[i], "-p") && i + 1 < argc) param = argv[++i];
        else if (!strcmp(argv[i], "-o") && i + 1 < argc) outp = argv[++i];
        else if (!strcmp(argv[i], "-maxit") && i + 1 < argc) maxit = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-times")) times = true;
    }
    if (!data) {
        fprintf(stderr, "usage: sdpa_port -ds data.dat-s [-p param] [-o out] [-maxit K] [-times]\n");
        return 2;
    }
    Solver S;
    if (param && !read_param(S.par, param)) {
        fprintf(stderr, "sdpa_port: cannot read %s\n", param);
        return 2;
    }
    mpf_set_default_prec(S.par.precision);
    S.eps = F(1.0);
    mpf_div_2exp(S.eps.v, S.eps.v, S.par.precision + 64);
    if (maxit >= 0 && maxit < S.par.maxIteration) S.par.maxIteration = maxit;
    if (!S.load(data)) {
        fprintf(stderr, "sdpa_port: cannot read %s\n", data);
        return 2;
    }
    FILE *out = outp ? fopen(outp, "w") : nullptr;
    auto t0 = std::chrono::steady_clock::now();
    S.initialize();
    if (times) fprintf(stderr, "SETUP %.6f\n", std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (out) fprintf(out, "   mu      thetaP  thetaD  objP      objD      alphaP  alphaD  beta \n");
    while (true) {
        auto a = std::chrono::steady_clock::now();
        const bool more = S.iterate(out);
        if (!more) break;
        if (times)
            fprintf(stderr, "ITER %d %.6f\n", S.iter - 1,
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count());
    }
    S.residuals();
    const int ph = S.phase;
    const int rev[] = {noINFO, dFEAS, pFEAS, pdFEAS, pdINF, pINF_dFEAS, pFEAS_dINF, pdOPT, dUNBD, pUNBD};
    FILE *fs[] = {out, stdout};
    for (FILE *f : fs) {
        if (!f) continue;
        S.print_iter(f);
        fprintf(f, "\nphase.value = %s\n   Iteration = %d\n", phase_names[rev[ph]], S.iter);
        fprintf(f, "          mu = %s\n", S.fmt("%4.16Fe", S.muCur).c_str());
        fprintf(f, "objValPrimal = %s\n", S.fmt("%10.16Fe", -S.objD).c_str());
        fprintf(f, "objValDual   = %s\n", S.fmt("%10.16Fe", -S.objP).c_str());
        fprintf(f, "p.feas.error = %s\n", S.fmt("%10.16Fe", S.normD).c_str());
        fprintf(f, "d.feas.error = %s\n", S.fmt("%10.16Fe", S.normP).c_str());
        fprintf(f, "total time   = %.3f\n",
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    if (out) fclose(out);
    return 0;
}
