// C ABI: problem construction, the whole interior-point solve, and the
// step-wise Newton / step-length / update entry points.
#include <string.h>

#include <algorithm>
#include <chrono>
#include <ctime>
#include <atomic>
#include <memory>
#include <thread>
#include <vector>

#include "capi_util.cuh"
#include "ml_host.h"
#include "problem.h"
#include "sdpg.h"
#include "solver.cuh"

using namespace sdpg;

struct sdpg_problem {
    RawProblem P;
};

struct sdpg_solver {
    std::unique_ptr<SolverBase> s;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    ~sdpg_solver() {
        s.reset();
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace {

Param to_param(const sdpg_param *p) {
    Param q;
    if (!p) return q;
    q.maxIteration = p->maxIteration;
    q.epsilonStar = p->epsilonStar;
    q.lambdaStar = p->lambdaStar;
    q.omegaStar = p->omegaStar;
    q.lowerBound = p->lowerBound;
    q.upperBound = p->upperBound;
    q.betaStar = p->betaStar;
    q.betaBar = p->betaBar;
    q.gammaStar = p->gammaStar;
    q.epsilonDash = p->epsilonDash;
    q.precision = p->precision;
    return q;
}

void from_param(const Param &q, sdpg_param *p) {
    p->maxIteration = q.maxIteration;
    p->epsilonStar = q.epsilonStar;
    p->lambdaStar = q.lambdaStar;
    p->omegaStar = q.omegaStar;
    p->lowerBound = q.lowerBound;
    p->upperBound = q.upperBound;
    p->betaStar = q.betaStar;
    p->betaBar = q.betaBar;
    p->gammaStar = q.gammaStar;
    p->epsilonDash = q.epsilonDash;
    p->precision = q.precision;
}

void check_param(const Param &q) {
    if (q.maxIteration < 0 || !(q.epsilonStar > 0) || !(q.lambdaStar > 0) || !(q.omegaStar > 1) ||
        q.betaStar < 0 || q.betaStar >= 1 || q.betaBar < 0 || q.betaBar >= 1 || q.betaStar > q.betaBar ||
        !(q.gammaStar > 0) || q.gammaStar >= 1 || !(q.epsilonDash > 0) || q.precision <= 0)
        throw sdpg_error(SDPG_ERR_ARG, "parameter out of its documented range (sdpa_parts.cpp:163-176)");
    if (q.precision > 512) throw sdpg_error(SDPG_ERR_ARG, "precision above 512 bits is not supported");
}

sdpg_solver *wrap(const RawProblem &P, const Param &q, int device, void *stream) {
    check_param(q);
    auto *h = new sdpg_solver();
    try {
        SDPG_CUDA(cudaSetDevice(device));
        if (stream) {
            h->stream = (cudaStream_t)stream;
        } else {
            SDPG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
            h->own_stream = true;
        }
        h->s.reset(make_solver(P, q, device, h->stream));
    } catch (...) {
        delete h;
        throw;
    }
    return h;
}

SolverBase &S(sdpg_solver *h) {
    if (!h || !h->s) throw sdpg_error(SDPG_ERR_ARG, "null solver handle");
    return *h->s;
}

// The reference driver's file output around the solve (main, sdpa_main.cpp:43-461):
// start line, the data file's title/comment lines (IO::read, sdpa_io.cpp:123-134), the
// file names, "DENSE computation" (Newton::initialize, sdpa_newton.cpp:349-350), the
// iteration table and summary, then parameters, time table, solution and final times.
int solve_file_impl(const char *data_path, bool data_dense, const Param &q, const char *param_path,
                    const char *init_path, bool init_sparse, const char *out_path, int device, FILE *display,
                    double *info12) {
    if (!data_path) throw sdpg_error(SDPG_ERR_ARG, "no data file");
    const auto t0 = std::chrono::steady_clock::now();
    std::string err;
    RawProblem P;
    if (!read_sdpa(data_path, data_dense, P, &err)) throw sdpg_error(SDPG_ERR_IO, err);
    InitPoint ip;
    const bool has_init = init_path && init_path[0];
    if (has_init && !read_init(init_path, init_sparse, P.m, P.blockStruct, ip, &err)) throw sdpg_error(SDPG_ERR_IO, err);
    const double read_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::unique_ptr<sdpg_solver> h(wrap(P, q, device, nullptr));
    if (has_init) h->s->set_initial_point(ip);
    FILE *out = nullptr;
    if (out_path && out_path[0]) {
        out = fopen(out_path, "w");
        if (!out) throw sdpg_error(SDPG_ERR_IO, std::string("cannot open out file ") + out_path);
    }
    int it;
    try {
        if (out) {
            const time_t now = time(nullptr);
            fprintf(out, "SDPA-GMP start at %s", ctime(&now));
            fputs(P.title.c_str(), out);
            fprintf(out, "data      is %s\n", data_path);
            if (param_path && param_path[0]) fprintf(out, "parameter is %s\n", param_path);
            if (has_init) fprintf(out, "initial   is %s\n", init_path);
            fprintf(out, "out       is %s\n", out_path);
            fprintf(out, "DENSE computation\n");
        }
        if (display) fprintf(display, "DENSE computations\n");
        it = h->s->run(out, display);
        if (out) {
            h->s->print_result_tail(out, read_s);
            const double loop = h->s->timers().total / 1000.0;
            fprintf(out, "    main loop time = %.6f\n", loop);
            fprintf(out, "        total time = %.6f\n",
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            fprintf(out, "  file   read time = %.6f\n", read_s);
        }
    } catch (...) {
        if (out) fclose(out);
        throw;
    }
    if (out) fclose(out);
    if (info12) h->s->info(info12);
    return it;
}

}  // namespace

extern "C" {

int sdpg_param_default(sdpg_param *p, int type) {
    return sdpg_guard([&] {
        if (!p) throw sdpg_error(SDPG_ERR_ARG, "null param");
        Param q;
        param_default(q, type);
        from_param(q, p);
        return (int)SDPG_OK;
    });
}

int sdpg_param_read(sdpg_param *p, const char *path) {
    return sdpg_guard([&] {
        if (!p || !path) throw sdpg_error(SDPG_ERR_ARG, "null argument");
        Param q = to_param(p);
        std::string err;
        if (!param_read(q, path, &err)) throw sdpg_error(SDPG_ERR_IO, err);
        from_param(q, p);
        return (int)SDPG_OK;
    });
}

sdpg_problem *sdpg_problem_new(int m, int nBlock, const int *blockStruct, int *err) {
    int rc = sdpg_guard([&] {
        if (m <= 0 || nBlock <= 0 || !blockStruct) throw sdpg_error(SDPG_ERR_ARG, "bad problem dimensions");
        for (int l = 0; l < nBlock; ++l)
            if (blockStruct[l] == 0) throw sdpg_error(SDPG_ERR_ARG, "zero block size");
        return (int)SDPG_OK;
    });
    if (err) *err = rc;
    if (rc != SDPG_OK) return nullptr;
    auto *p = new sdpg_problem();
    p->P.m = m;
    p->P.blockStruct.assign(blockStruct, blockStruct + nBlock);
    p->P.c.assign(m, ml_zero<16>());
    return p;
}

sdpg_problem *sdpg_problem_read(const char *path, int dense_format, int *err) {
    auto *p = new sdpg_problem();
    int rc = sdpg_guard([&] {
        std::string e;
        if (!path || !read_sdpa(path, dense_format != 0, p->P, &e)) throw sdpg_error(SDPG_ERR_IO, e);
        return (int)SDPG_OK;
    });
    if (err) *err = rc;
    if (rc != SDPG_OK) {
        delete p;
        return nullptr;
    }
    return p;
}

void sdpg_problem_free(sdpg_problem *p) { delete p; }

int sdpg_problem_set_c(sdpg_problem *p, int k, const char *text) {
    return sdpg_guard([&] {
        if (!p || k < 1 || k > p->P.m || !text) throw sdpg_error(SDPG_ERR_ARG, "bad c index");
        mlf<16> v;
        if (!ml_parse<16>(text, &v)) throw sdpg_error(SDPG_ERR_ARG, "not a number");
        p->P.c[k - 1] = v;
        return (int)SDPG_OK;
    });
}

int sdpg_problem_set_c_double(sdpg_problem *p, int k, double v) {
    return sdpg_guard([&] {
        if (!p || k < 1 || k > p->P.m) throw sdpg_error(SDPG_ERR_ARG, "bad c index");
        p->P.c[k - 1] = ml_from_double<16>(v);
        return (int)SDPG_OK;
    });
}

int sdpg_problem_add_dense(sdpg_problem *p, int k, int block, int n, const double *A) {
    return sdpg_guard([&] {
        if (!p || !A || k < 0 || k > p->P.m || block < 1 || block > (int)p->P.blockStruct.size())
            throw sdpg_error(SDPG_ERR_ARG, "entry index out of range");
        const int bs = p->P.blockStruct[block - 1];
        if (bs < 0 || n != bs) throw sdpg_error(SDPG_ERR_ARG, "n must equal the (SDP) block size");
        p->P.entries.reserve(p->P.entries.size() + (size_t)n * (n + 1) / 2);
        for (int b = 0; b < n; ++b)
            for (int a = 0; a <= b; ++a) {
                RawEntry e;
                e.k = k;
                e.block = block - 1;
                e.i = a;
                e.j = b;
                e.v = ml_from_double<16>(A[a + (size_t)b * n]);
                p->P.entries.push_back(e);
            }
        return (int)SDPG_OK;
    });
}

int sdpg_problem_add_entry(sdpg_problem *p, int k, int block, int i, int j, const char *text) {
    return sdpg_guard([&] {
        if (!p || !text || k < 0 || k > p->P.m || block < 1 || block > (int)p->P.blockStruct.size())
            throw sdpg_error(SDPG_ERR_ARG, "entry index out of range");
        const int bs = p->P.blockStruct[block - 1];
        const int size = bs < 0 ? -bs : bs;
        if (i < 1 || j < 1 || i > size || j > size) throw sdpg_error(SDPG_ERR_ARG, "out of range in input data");
        RawEntry e;
        if (!ml_parse<16>(text, &e.v)) throw sdpg_error(SDPG_ERR_ARG, "not a number");
        e.k = k;
        e.block = block - 1;
        e.i = i - 1;
        e.j = j - 1;
        p->P.entries.push_back(e);
        return (int)SDPG_OK;
    });
}

int sdpg_problem_add_entry_mpf(sdpg_problem *p, int k, int block, int i, int j, const sdpg_mpf_t *v) {
    return sdpg_guard([&] {
        if (!p || !v) throw sdpg_error(SDPG_ERR_ARG, "null argument");
        if (k < 0 || k > p->P.m || block < 1 || block > (int)p->P.blockStruct.size())
            throw sdpg_error(SDPG_ERR_ARG, "entry index out of range");
        const int bs = p->P.blockStruct[block - 1];
        const int size = bs < 0 ? -bs : bs;
        if (i < 1 || j < 1 || i > size || j > size) throw sdpg_error(SDPG_ERR_ARG, "out of range in input data");
        RawEntry e;
        e.v = ml_from_mpf<16>(v->_mp_size, v->_mp_exp, v->_mp_d);
        e.k = k;
        e.block = block - 1;
        e.i = i - 1;
        e.j = j - 1;
        p->P.entries.push_back(e);
        return (int)SDPG_OK;
    });
}

sdpg_solver *sdpg_solver_create(const sdpg_problem *p, const sdpg_param *param, int device, void *stream, int *err) {
    sdpg_solver *h = nullptr;
    int rc = sdpg_guard([&] {
        if (!p) throw sdpg_error(SDPG_ERR_ARG, "null problem");
        Param q = param ? to_param(param) : Param();
        h = wrap(p->P, q, device, stream);
        return (int)SDPG_OK;
    });
    if (err) *err = rc;
    return rc == SDPG_OK ? h : nullptr;
}

void sdpg_solver_destroy(sdpg_solver *h) { delete h; }

int sdpg_solver_limbs(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).limbs(); });
}

int sdpg_solver_initialize(sdpg_solver *h) {
    return sdpg_guard([&] {
        S(h).initialize();
        return (int)SDPG_OK;
    });
}

int sdpg_solver_run(sdpg_solver *h, const char *out_path, int print_to_stdout) {
    return sdpg_guard([&] {
        FILE *out = nullptr;
        if (out_path && out_path[0]) {
            out = fopen(out_path, "w");
            if (!out) throw sdpg_error(SDPG_ERR_IO, std::string("cannot open out file ") + out_path);
        }
        int it;
        try {
            it = S(h).run(out, print_to_stdout ? stdout : nullptr);
        } catch (...) {
            if (out) fclose(out);
            throw;
        }
        if (out) fclose(out);
        return it;
    });
}

int sdpg_solver_iterate(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).iterate(nullptr); });
}

int sdpg_newton(sdpg_solver *h, int direction) {
    return sdpg_guard([&] { return S(h).newton(direction) ? (int)SDPG_OK : (int)SDPG_ERR_NOT_PD; });
}

int sdpg_step_length(sdpg_solver *h, int direction) {
    return sdpg_guard([&] {
        S(h).step_length(direction);
        return (int)SDPG_OK;
    });
}

int sdpg_loop_phase_check(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).loop_phase_check() ? 1 : 0; });
}

int sdpg_loop_direction(sdpg_solver *h, int corrector) {
    return sdpg_guard([&] {
        S(h).loop_direction(corrector);
        return (int)SDPG_OK;
    });
}

int sdpg_loop_corrector_break(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).loop_corrector_break() ? 1 : 0; });
}

int sdpg_loop_record(sdpg_solver *h, void *out_file, void *display_file) {
    return sdpg_guard([&] {
        S(h).loop_record((FILE *)out_file, (FILE *)display_file);
        return (int)SDPG_OK;
    });
}

int sdpg_loop_update(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).loop_update() ? (int)SDPG_OK : (int)SDPG_ERR_NOT_PD; });
}

int sdpg_loop_after_update(sdpg_solver *h) {
    return sdpg_guard([&] {
        S(h).loop_after_update();
        return (int)SDPG_OK;
    });
}

int sdpg_loop_finish(sdpg_solver *h, void *out_file, void *display_file) {
    return sdpg_guard([&] {
        S(h).loop_finish((FILE *)out_file, (FILE *)display_file);
        return (int)SDPG_OK;
    });
}

int sdpg_loop_values(sdpg_solver *h, int *phase, int *iteration, void *out_ml9) {
    return sdpg_guard([&] {
        if (!phase || !iteration || !out_ml9) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).loop_values(phase, iteration, out_ml9);
        return (int)SDPG_OK;
    });
}

int sdpg_update(sdpg_solver *h) {
    return sdpg_guard([&] { return S(h).update() ? (int)SDPG_OK : (int)SDPG_ERR_NOT_PD; });
}

int sdpg_residuals(sdpg_solver *h) {
    return sdpg_guard([&] {
        S(h).residuals();
        return (int)SDPG_OK;
    });
}

int sdpg_solution_info(sdpg_solver *h, double *out12) {
    return sdpg_guard([&] {
        if (!out12) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).info(out12);
        return (int)SDPG_OK;
    });
}

int sdpg_solution_text(sdpg_solver *h, int which, int digits, char *buf, int cap) {
    return sdpg_guard([&] {
        std::string s = S(h).info_text(which, digits > 1 ? digits : 2);
        if (!buf || (int)s.size() + 1 > cap) throw sdpg_error(SDPG_ERR_ARG, "buffer too small");
        memcpy(buf, s.c_str(), s.size() + 1);
        return (int)SDPG_OK;
    });
}

int sdpg_get_xvec(sdpg_solver *h, int form, void *out) {
    return sdpg_guard([&] {
        if (!out) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).get_y(out, form);
        return (int)SDPG_OK;
    });
}

int sdpg_get_block(sdpg_solver *h, int which, int block, int form, void *out) {
    return sdpg_guard([&] {
        if (!out || block < 0 || block >= S(h).nblocks()) throw sdpg_error(SDPG_ERR_ARG, "bad block");
        S(h).get_block(which, block, out, form);
        return (int)SDPG_OK;
    });
}

int sdpg_make_schur(sdpg_solver *h, void *out_ml) {
    return sdpg_guard([&] {
        if (!out_ml) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).make_bmat(out_ml);
        return (int)SDPG_OK;
    });
}

int sdpg_make_gvec(sdpg_solver *h, int direction, void *out_ml) {
    return sdpg_guard([&] {
        if (!out_ml) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).make_gvec(direction, out_ml);
        return (int)SDPG_OK;
    });
}

int sdpg_min_eigen(sdpg_solver *h, int side, void *out_ml) {
    return sdpg_guard([&] {
        if (!out_ml) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).min_eigen(side, out_ml);
        return (int)SDPG_OK;
    });
}

int sdpg_get_vector(sdpg_solver *h, int which, void *out_ml) {
    return sdpg_guard([&] {
        if (!out_ml) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).get_vec(which, out_ml);
        return (int)SDPG_OK;
    });
}

int sdpg_solver_dims(sdpg_solver *h, int *m, int *nblocks, int *block_sizes, int cap) {
    return sdpg_guard([&] {
        SolverBase &s = S(h);
        if (m) *m = s.m();
        if (nblocks) *nblocks = s.nblocks();
        for (int l = 0; block_sizes && l < s.nblocks() && l < cap; ++l) block_sizes[l] = s.block_size(l);
        return (int)SDPG_OK;
    });
}

int sdpg_solver_timers(sdpg_solver *h, double *out8) {
    return sdpg_guard([&] {
        const Timers &t = S(h).timers();
        double v[8] = {t.schur, t.cholesky, t.rmat_gvec, t.dxdz, t.steplen, t.update, t.residual, t.total};
        memcpy(out8, v, sizeof v);
        return (int)SDPG_OK;
    });
}

int sdpg_solver_history(sdpg_solver *h, double *out, int cap) {
    return sdpg_guard([&] {
        const auto &hist = S(h).history();
        const int n = (int)hist.size();
        for (int i = 0; i < n && i < cap; ++i) {
            const IterRecord &r = hist[i];
            double v[9] = {(double)r.it, r.mu, r.thetaP, r.thetaD, r.objP, r.objD, r.alphaP, r.alphaD, r.beta};
            memcpy(out + 9 * i, v, sizeof v);
        }
        return n;
    });
}

long long sdpg_solver_gemm_macs(sdpg_solver *h) {
    long long v = 0;
    int rc = sdpg_guard([&] {
        v = S(h).gemm_macs();
        return (int)SDPG_OK;
    });
    return rc == SDPG_OK ? v : rc;
}

int sdpg_solver_gemm_profile(sdpg_solver *h, int enable, double *out3) {
    return sdpg_guard([&] {
        if (out3) S(h).gemm_profile(out3);
        if (enable >= 0) S(h).set_gemm_profiling(enable != 0);
        return (int)SDPG_OK;
    });
}

int sdpg_solver_io_bytes(sdpg_solver *h, long long *h2d, long long *d2h) {
    return sdpg_guard([&] {
        long long a = 0, b = 0;
        S(h).io_bytes(&a, &b);
        if (h2d) *h2d = a;
        if (d2h) *d2h = b;
        return (int)SDPG_OK;
    });
}

int sdpg_solver_reset_counters(sdpg_solver *h) {
    return sdpg_guard([&] {
        S(h).reset_counters();
        return (int)SDPG_OK;
    });
}

int sdpg_solver_read_initial_point(sdpg_solver *h, const char *path, int sparse) {
    return sdpg_guard([&] {
        SolverBase &s = S(h);
        InitPoint ip;
        std::string err;
        if (!path || !read_init(path, sparse != 0, s.m(), s.block_structure(), ip, &err))
            throw sdpg_error(SDPG_ERR_IO, path ? err : std::string("no init file"));
        s.set_initial_point(ip);
        return SDPG_OK;
    });
}

int sdpg_solver_set_policy(sdpg_solver *h, sdpg_policy *p, int flags) {
    return sdpg_guard([&] {
        if (flags < 0 || flags > 3) throw sdpg_error(SDPG_ERR_ARG, "policy flags are 0..3");
        S(h).set_policy(p ? &p->p : nullptr, flags);
        return SDPG_OK;
    });
}

int sdpg_solver_policy_stats(sdpg_solver *h, double *out4) {
    return sdpg_guard([&] {
        if (!out4) throw sdpg_error(SDPG_ERR_ARG, "null output");
        S(h).policy_stats(out4);
        return SDPG_OK;
    });
}

int sdpg_solver_features(sdpg_solver *h, float *out, int cap) {
    return sdpg_guard([&] {
        const auto &f = S(h).features();
        const int rows = (int)f.size();
        if (out)
            for (int r = 0; r < std::min(rows, cap); ++r)
                for (int i = 0; i < kPolIn; ++i) out[(size_t)r * kPolIn + i] = f[r][i];
        return rows;
    });
}

int sdpg_solve_file(const char *data_path, const char *param_path, const char *out_path, int device, double *info12) {
    return sdpg_guard([&] {
        Param q;
        std::string err;
        if (param_path && param_path[0] && !param_read(q, param_path, &err)) throw sdpg_error(SDPG_ERR_IO, err);
        return solve_file_impl(data_path, false, q, param_path, nullptr, false, out_path, device, nullptr, info12);
    });
}

int sdpg_solve_file_ex(const char *data_path, int data_dense, const sdpg_param *param, const char *param_path,
                       const char *init_path, int init_sparse, const char *out_path, int device, int print_to_stdout,
                       double *info12) {
    return sdpg_guard([&] {
        Param q = to_param(param);
        std::string err;
        if (!param && param_path && param_path[0] && !param_read(q, param_path, &err))
            throw sdpg_error(SDPG_ERR_IO, err);
        return solve_file_impl(data_path, data_dense != 0, q, param_path, init_path, init_sparse != 0, out_path,
                               device, print_to_stdout ? stdout : nullptr, info12);
    });
}

int sdpg_solve_batch(int count, sdpg_problem *const *problems, const sdpg_param *param, int device, int concurrency,
                     double *info12, int *iterations) {
    return sdpg_guard([&] {
        if (count < 0 || (count > 0 && !problems) || concurrency < 1)
            throw sdpg_error(SDPG_ERR_ARG, "bad batch arguments");
        for (int i = 0; i < count; ++i)
            if (!problems[i]) throw sdpg_error(SDPG_ERR_ARG, "null problem in batch");
        const Param q = param ? to_param(param) : Param();
        check_param(q);
        std::atomic<int> next{0}, solved{0};
        auto worker = [&]() {
            if (cudaSetDevice(device) != cudaSuccess) return;
            for (;;) {
                const int i = next.fetch_add(1);
                if (i >= count) break;
                int its;
                try {
                    // each solver owns its streams and scratch: solvers on different
                    // host threads run concurrently on the GPU
                    std::unique_ptr<sdpg_solver> h(wrap(problems[i]->P, q, device, nullptr));
                    its = h->s->run(nullptr, nullptr);
                    if (info12) h->s->info(info12 + 12 * (size_t)i);
                    solved.fetch_add(1);
                } catch (const sdpg_error &e) {
                    set_last_error(e.what());
                    its = e.code;
                } catch (const std::exception &e) {
                    set_last_error(e.what());
                    its = SDPG_ERR_ARG;
                }
                if (iterations) iterations[i] = its;
            }
        };
        const int nt = std::min(concurrency, std::max(count, 1));
        std::vector<std::thread> threads;
        threads.reserve(nt);
        for (int t = 0; t < nt; ++t) threads.emplace_back(worker);
        for (auto &t : threads) t.join();
        return solved.load();
    });
}

}  // extern "C"
