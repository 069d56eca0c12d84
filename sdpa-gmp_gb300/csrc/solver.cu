// Interior-point solver: state resident on the GPU, control scalars on the host.
//
// Each method restates the reference routine named in its comment.  The
// reference is SDPA-GMP 7.1.3 with REVERSE_PRIMAL_DUAL on (sdpa_tool.h:84):
// internally it solves  min C.X  s.t. A_i.X = b_i, X >= 0  (C = -F0 of the
// file) with the HRVW/KSH/M direction and Mehrotra predictor-corrector steps.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <utility>

#include "solver.cuh"

namespace sdpg {

const char *phase_name(int phase) {
    switch (phase) {
        case noINFO: return "noINFO    ";
        case pFEAS: return "pFEAS     ";
        case dFEAS: return "dFEAS     ";
        case pdFEAS: return "pdFEAS    ";
        case pdINF: return "pdINF     ";
        case pFEAS_dINF: return "pFEAS_dINF";
        case pINF_dFEAS: return "pINF_dFEAS";
        case pdOPT: return "pdOPT     ";
        case pUNBD: return "pUNBD     ";
        case dUNBD: return "dUNBD     ";
    }
    return "phase error";
}

namespace {

enum Formula { F1 = 0, F2 = 1, F3 = 2 };

template <int N>
class Solver final : public SolverBase {
    using R = Real<N>;
    using V = mlf<N>;

    struct Blk {
        int n = 0;
        V *C, *X, *Z, *Zinv, *LX, *LZ, *Dx, *Dz, *Rm, *XRDZ, *W1, *W2, *Dres, *Lt, *F;
        // Lanczos vectors and tridiagonal storage, one set per side (0: X, 1: Z)
        V *q[2], *qold[2], *r[2], *w[2], *tmp[2], *td[2], *te[2], *sl[2];
        V *Mop[2] = {nullptr, nullptr}, *Mtmp[2] = {nullptr, nullptr};  // L X L^T of a Lanczos run (n > 20)
        int *lzctl[2] = {nullptr, nullptr};  // device loop flags of a Lanczos run: [0] going on, [1] steps done
        V *SW1 = nullptr, *SW2 = nullptr;  // Z-side work matrices of the small-block eigenvalue path
        BlockDev<N> cons;
        std::vector<int> f1_owners_h;
        int *f1_owners = nullptr;
        int nF1 = 0;
        int lanczos_kmax = 0;
        // An LP block of the file (negative size, or size 1), held as a diagonal n x n
        // block: the same iterates, Schur entries and residuals as the reference's LP
        // arithmetic, since every product of diagonal matrices stays exactly diagonal;
        // its step length uses the LP rule instead of Lanczos.
        bool lp = false;
    };

  public:
    Solver(const RawProblem &P, const Param &par, int device, cudaStream_t stream)
        : par_(par), lambda_default_(par.lambdaStar), dev_(device), st_(stream) {
        SDPG_CUDA(cudaSetDevice(device));
        if (!st_) throw sdpg_error(SDPG_ERR_ARG, "the solver needs a stream");
        keep_pool_memory(device);
        ws_.stream = st_;
        ws2_.stream = st_;
        setup(P);
        SDPG_CUDA(cudaStreamSynchronize(st_));  // allocations and uploads complete
    }
    // Device memory goes back to the stream-ordered pool on the main stream once both
    // streams are idle: no device-wide synchronisation, so concurrent solvers keep running.
    ~Solver() override {
        cudaStreamSynchronize(st_);
        if (st2_) cudaStreamSynchronize(st2_);
        if (st2_) cudaStreamDestroy(st2_);
        if (ev_fork_) cudaEventDestroy(ev_fork_);
        if (ev_join_) cudaEventDestroy(ev_join_);
        pinned_release(pinned_, kPinned * sizeof(V));
        for (void *p : allocs_) cudaFreeAsync(p, st_);
        ws_.release();
        ws2_.release();
        for (auto &e : ev_) cudaEventDestroy(e);
        for (auto &e : prof_ev_) cudaEventDestroy(e);
    }

    int limbs() const override { return N; }
    int m() const override { return m_; }
    int nblocks() const override { return (int)blk_.size(); }
    int block_size(int l) const override { return blk_[l].n; }
    int phase() const override { return phase_; }
    int iteration() const override { return iter_; }
    const Timers &timers() const override { return tm_; }
    const std::vector<IterRecord> &history() const override { return hist_; }
    void set_trace(FILE *f) override { trace_ = f; }
    long long gemm_macs() const override { return gemm_macs_; }
    void reset_counters() override {
        gemm_macs_ = 0;
        tm_ = Timers();
        collect_gemm_events();
        prof_ms_ = 0;
        prof_launches_ = 0;
        prof_macs_ = 0;
    }
    void set_gemm_profiling(bool on) override { prof_on_ = on; }
    void collect_gemm_events() {
        if (prof_used_ == 0) return;
        SDPG_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < prof_used_; ++i) {
            float ms = 0;
            SDPG_CUDA(cudaEventElapsedTime(&ms, prof_ev_[2 * i], prof_ev_[2 * i + 1]));
            prof_ms_ += ms;
        }
        prof_used_ = 0;
    }
    void gemm_profile(double *o) override {
        collect_gemm_events();
        o[0] = prof_ms_;
        o[1] = (double)prof_launches_;
        o[2] = (double)prof_macs_;
    }
    void io_bytes(long long *h2d, long long *d2h) const override {
        *h2d = h2d_;
        *d2h = d2h_;
    }
    void sync() override { SDPG_CUDA(cudaStreamSynchronize(st_)); }

    // ---------------------------------------------------------------- learned proposal

    void set_policy(const Policy *p, int flags) override {
        if (p && p->device != dev_) throw sdpg_error(SDPG_ERR_ARG, "the policy lives on another device");
        if (p && !pol_dev_) pol_dev_ = (float *)dalloc_raw(16 * sizeof(float));
        policy_ = p;
        pol_flags_ = p ? flags : 0;
    }
    void policy_stats(double *o) const override {
        o[0] = (double)pol_props_;
        o[1] = (double)pol_fallbacks_;
        o[2] = par_.lambdaStar;
        o[3] = pol_lambda_prop_;
    }
    const std::vector<std::array<float, kPolIn>> &features() const override { return feats_; }

    // log10 mu, log10 primal / dual residual max-norms, previous step lengths, the rule's beta
    std::array<float, kPolIn> policy_features(const R &beta_rule) const {
        auto lg = [](const R &v) {
            const double d = fabs(v.d());
            return (float)log10(d > 1e-40 ? d : 1e-40);
        };
        return {lg(muCur_), lg(normP_), lg(normD_), (float)lastAP_.d(), (float)lastAD_.d(), (float)beta_rule.d()};
    }
    void policy_eval(const std::array<float, kPolIn> &f, float y[kPolOut]) {
        float *h = reinterpret_cast<float *>(pinned_ + kPinned - 4);  // 4 spare slots at the end
        for (int i = 0; i < kPolIn; ++i) h[i] = f[i];
        h2d_ += kPolIn * (long long)sizeof(float);
        d2h_ += kPolOut * (long long)sizeof(float);
        SDPG_CUDA(cudaMemcpyAsync(pol_dev_, h, kPolIn * sizeof(float), cudaMemcpyHostToDevice, st_));
        policy_forward_device(*policy_, pol_dev_, 1, pol_dev_ + 8, st_);
        SDPG_CUDA(cudaMemcpyAsync(h + 8, pol_dev_ + 8, kPolOut * sizeof(float), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        for (int o = 0; o < kPolOut; ++o) y[o] = h[8 + o];
    }
    // the checks a proposed corrector must pass: the predicted mu falls by at least a
    // quarter of the shorter step, and a residual that is not yet zero is reduced by a
    // step of at least one half
    bool proposal_ok() {
        const R xMatvMat = ip_blocks(&Blk::X, &Blk::Dz);
        const R uMatzMat = ip_blocks(&Blk::Dx, &Blk::Z);
        const R uMatvMat = ip_blocks(&Blk::Dx, &Blk::Dz);
        const R muNew = muCur_ + (aP_ * uMatzMat + aD_ * xMatvMat + aP_ * aD_ * uMatvMat) / R(nDim_);
        if (!(muNew <= (R(1.0) - R(0.25) * rmin(aP_, aD_)) * muCur_)) return false;
        const bool primal_open = phase_ == noINFO || phase_ == dFEAS;
        const bool dual_open = phase_ == noINFO || phase_ == pFEAS;
        if (primal_open && aP_ < R(0.5)) return false;
        if (dual_open && aD_ < R(0.5)) return false;
        return true;
    }

    // ---------------------------------------------------------------- setup

    void setup(const RawProblem &P) {
        m_ = P.m;
        if (m_ <= 0) throw sdpg_error(SDPG_ERR_ARG, "mDIM must be positive");
        std::vector<int> sdp_of_file(P.blockStruct.size(), -1);
        for (size_t l = 0; l < P.blockStruct.size(); ++l) {
            const int bs = P.blockStruct[l];
            if (bs == 0) throw sdpg_error(SDPG_ERR_ARG, "block size 0");
            // main, sdpa_main.cpp:113-129: size >= 2 is an SDP block, negative or 1 an LP block
            sdp_of_file[l] = (int)blk_.size();
            blk_.emplace_back();
            blk_.back().n = bs < 0 ? -bs : bs;
            blk_.back().lp = bs < 2;
        }
        nDim_ = 0;
        for (auto &b : blk_) nDim_ += b.n;
        // b = c
        std::vector<V> bh(m_);
        for (int k = 0; k < m_; ++k) bh[k] = narrow<N>(P.c[k]);
        b_ = dalloc(m_);
        y_ = dalloc(m_);
        Dy_ = dalloc(m_);
        g_ = dalloc(m_);
        p_ = dalloc(m_);
        B_ = dalloc((size_t)m_ * m_);
        BLinv_ = dalloc((size_t)m_ * m_);
        BLinvT_ = dalloc((size_t)m_ * m_);
        Dytmp_ = dalloc(m_);
        upload(b_, bh.data(), m_);
        b_h_ = bh;
        info_ = (int *)dalloc_raw(64);
        status_ = (int *)dalloc_raw(64);
        slot_ = dalloc(kSlots);
        // entries per (constraint, block)
        const int nb = (int)blk_.size();
        std::vector<std::vector<std::vector<const RawEntry *>>> ent(m_ + 1, std::vector<std::vector<const RawEntry *>>(nb));
        for (const auto &e : P.entries) {
            const int l = sdp_of_file[e.block];
            if (l < 0) continue;
            ent[e.k][l].push_back(&e);
        }
        size_t max_ws = 0;
        const mlf<N> kappa_v = ml_from_double<N>(1.2);  // Newton::computeFormula_SDP(..., KAPPA), sdpa_main.cpp:27
        for (int l = 0; l < nb; ++l) {
            Blk &B = blk_[l];
            const int n = B.n;
            const size_t nn = (size_t)n * n;
            V **mats[] = {&B.C, &B.X, &B.Z, &B.Zinv, &B.LX, &B.LZ, &B.Dx, &B.Dz, &B.Rm, &B.XRDZ, &B.W1, &B.W2, &B.Dres, &B.Lt, &B.F};
            for (V **mp : mats) *mp = dalloc(nn);
            // C = -F0 (dense on the device; duplicates accumulate like sparse inner products)
            {
                std::vector<V> Ch(nn, ml_zero<N>());
                for (const RawEntry *e : ent[0][l]) {
                    const V v = ml_neg(narrow<N>(e->v));
                    Ch[e->i + (size_t)n * e->j] = ml_add(Ch[e->i + (size_t)n * e->j], v);
                    if (e->i != e->j) Ch[e->j + (size_t)n * e->i] = ml_add(Ch[e->j + (size_t)n * e->i], v);
                }
                upload(B.C, Ch.data(), nn);
            }
            // constraints touching this block, in increasing index (InputData::initialize_index_SDP)
            std::vector<int> cids, nzc, nze, dense;
            for (int k = 1; k <= m_; ++k) {
                if (ent[k][l].empty()) continue;
                cids.push_back(k - 1);
                const int cnt = (int)ent[k][l].size();
                nzc.push_back(cnt);
                // SparseMatrix::changeToDense: stays sparse if NonZeroCount < nRow*nCol*0.20
                const bool isdense = !((double)cnt < (double)(n * n) * 0.20);
                dense.push_back(isdense ? 1 : 0);
                int eff = 0;
                if (isdense) eff = n * n;
                else
                    for (const RawEntry *e : ent[k][l]) eff += (e->i == e->j) ? 1 : 2;
                nze.push_back(eff);
            }
            const int nc = (int)cids.size();
            B.cons.n = n;
            B.cons.nc = nc;
            // formula choice (Newton::computeFormula_SDP, sdpa_newton.cpp:694-819)
            std::vector<int> formula(nc);
            for (int a = 0; a < nc; ++a) {
                const int i = cids[a], inz = nze[a];
                long up = inz;
                for (int c = 0; c < nc; ++c) {
                    const int j = cids[c], jnz = nze[c];
                    if (jnz < inz) up += jnz;
                    else if (jnz == inz && j < i) up += jnz;
                }
                const R K(kappa_v), nR(n), inzR(inz), upR(up);
                const R f1 = K * nR * inzR + nR * nR * nR + K * upR;
                const R f2 = K * nR * inzR + K * (nR + R(1)) * upR;
                const R f3 = K * (R(2) * K * inzR + R(1)) * upR / K;
                if (dense[a]) formula[a] = (f1 < f2) ? F1 : F2;
                else if (f1 < f2 && f1 < f3) formula[a] = F1;
                else if (f2 < f3) formula[a] = F2;
                else formula[a] = F3;
            }
            // rank by (NonZeroEffect, index)
            std::vector<int> order(nc), rank(nc);
            for (int a = 0; a < nc; ++a) order[a] = a;
            std::sort(order.begin(), order.end(), [&](int x, int y) {
                return nze[x] != nze[y] ? nze[x] < nze[y] : cids[x] < cids[y];
            });
            for (int r = 0; r < nc; ++r) rank[order[r]] = r;
            // sparse COO (symmetric expansion, duplicates merged) and dense matrices
            std::vector<int> sp_off(nc + 1, 0), sp_row, sp_col, dn_slot(nc, -1), dn_cid, dn_local;
            std::vector<V> sp_val, dn_val;
            std::map<long long, std::vector<std::pair<int, V>>> pos;  // r + c*n -> (k, v)
            for (int a = 0; a < nc; ++a) {
                const auto &E = ent[cids[a] + 1][l];
                if (dense[a]) {
                    dn_slot[a] = (int)dn_cid.size();
                    dn_cid.push_back(cids[a]);
                    dn_local.push_back(a);
                    std::vector<V> M(nn, ml_zero<N>());
                    for (const RawEntry *e : E) {  // changeToDense: later duplicates overwrite
                        const V v = narrow<N>(e->v);
                        M[e->i + (size_t)n * e->j] = v;
                        M[e->j + (size_t)n * e->i] = v;
                    }
                    dn_val.insert(dn_val.end(), M.begin(), M.end());
                } else {
                    std::map<long long, V> acc;
                    for (const RawEntry *e : E) {
                        const V v = narrow<N>(e->v);
                        const long long k1 = e->i + (long long)n * e->j;
                        acc[k1] = acc.count(k1) ? ml_add(acc[k1], v) : v;
                        if (e->i != e->j) {
                            const long long k2 = e->j + (long long)n * e->i;
                            acc[k2] = acc.count(k2) ? ml_add(acc[k2], v) : v;
                        }
                    }
                    for (auto &kv : acc) {
                        sp_row.push_back((int)(kv.first % n));
                        sp_col.push_back((int)(kv.first / n));
                        sp_val.push_back(kv.second);
                        pos[kv.first].push_back({cids[a], kv.second});
                    }
                }
                sp_off[a + 1] = (int)sp_row.size();
            }
            B.cons.ndense = (int)dn_cid.size();
            B.cons.cid = upload_new(cids);
            B.cons.rank = upload_new(rank);
            B.cons.formula = upload_new(formula);
            B.cons.sp_off = upload_new(sp_off);
            B.cons.sp_row = upload_new(sp_row);
            B.cons.sp_col = upload_new(sp_col);
            B.cons.sp_val = upload_new(sp_val);
            B.cons.dn_slot = upload_new(dn_slot);
            B.cons.dn_cid = upload_new(dn_cid);
            B.cons.dn_local = upload_new(dn_local);
            std::vector<long long> dn_off(dn_cid.size());
            for (size_t d = 0; d < dn_off.size(); ++d) dn_off[d] = (long long)d * (long long)nn;
            B.cons.dn_off = upload_new(dn_off);
            B.cons.dense = upload_new(dn_val);
            std::vector<int> pos_rc, pos_off(1, 0), pos_k;
            std::vector<V> pos_v;
            for (auto &kv : pos) {
                pos_rc.push_back((int)kv.first);
                for (auto &pr : kv.second) {
                    pos_k.push_back(pr.first);
                    pos_v.push_back(pr.second);
                }
                pos_off.push_back((int)pos_k.size());
            }
            B.cons.npos = (int)pos_rc.size();
            B.cons.pos_rc = upload_new(pos_rc);
            B.cons.pos_off = upload_new(pos_off);
            B.cons.pos_k = upload_new(pos_k);
            B.cons.pos_v = upload_new(pos_v);
            for (int a = 0; a < nc; ++a)
                if (formula[a] != F3) B.f1_owners_h.push_back(a);
            B.nF1 = (int)B.f1_owners_h.size();
            B.f1_owners = upload_new(B.f1_owners_h);
            // Lanczos vectors; at most min(n, sqrt(n)+10) steps (sdpa_linear.cpp:43)
            B.lanczos_kmax = std::min(n, (int)sqrt((double)n) + 12) + 2;
            for (int side = 0; side < 2; ++side) {
                B.q[side] = dalloc(n);
                B.qold[side] = dalloc(n);
                B.r[side] = dalloc(n);
                B.w[side] = dalloc(n);
                B.tmp[side] = dalloc(n);
                B.td[side] = dalloc(std::max(B.lanczos_kmax, n) + 2);
                B.te[side] = dalloc(std::max(B.lanczos_kmax, n) + 2);
                B.sl[side] = dalloc(16);
                B.lzctl[side] = (int *)dalloc_raw(16);
            }
            if (B.lp) {
                // no eigenvalue work space: the LP rule reads the diagonals
            } else if (n <= 20) {
                B.SW1 = dalloc(nn);
                B.SW2 = dalloc(nn);
            } else {
                for (int side = 0; side < 2; ++side) {
                    B.Mop[side] = dalloc(nn);
                    B.Mtmp[side] = dalloc(nn);
                }
            }
            // workspace need
            max_ws = std::max(max_ws, gemm_bytes(n, n, n, 1));
            const int chunk = f1_chunk(B);
            if (B.nF1 > 0) {
                max_ws = std::max(max_ws, gemm_bytes(n, n, n, chunk) + 3 * (size_t)chunk * nn * sizeof(V));
                if (B.cons.ndense > 0) {
                    max_ws = std::max(max_ws, gemm_bytes(chunk, B.cons.ndense, (int)nn, 1) +
                                                  3 * (size_t)chunk * nn * sizeof(V) +
                                                  (size_t)chunk * B.cons.ndense * sizeof(V) + (size_t)chunk * B.cons.ndense * 16);
                }
            }
            max_ws = std::max(max_ws, gemm_bytes(32, n, n, 1) + 32 * (size_t)n * sizeof(V));
            max_ws = std::max(max_ws, ml_trtri_workspace_bytes<N>(n));
            max_ws = std::max(max_ws, ml_potrf_workspace_bytes<N>(n));
        }
        max_ws = std::max(max_ws, gemm_bytes(m_, m_, 32, 1));
        max_ws = std::max(max_ws, gemm_bytes(m_, 32, m_, 1));  // left-looking Cholesky panel update
        max_ws = std::max(max_ws, ml_trtri_workspace_bytes<N>(m_));
        max_ws = std::max(max_ws, ml_potrf_workspace_bytes<N>(m_));
        ws_.reserve(max_ws + (64u << 20));
        ws2_.reserve(max_ws + (64u << 20));
        // this solver's own time-out word (zeroed by dalloc_raw) for the bounded waits of its
        // tensor-core GEMMs and Cholesky panels: a wait that gives up in another solver on
        // the device does not fail this one
        tc_error_ = (int *)dalloc_raw(sizeof(int));
        ws_.error = ws2_.error = tc_error_;
        SDPG_CUDA(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
        SDPG_CUDA(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
        SDPG_CUDA(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
        pinned_ = (V *)pinned_acquire(kPinned * sizeof(V));
        info2_ = (int *)dalloc_raw(sizeof(int) * (4 * blk_.size() + 16));
        info_all_ = (int *)dalloc_raw(sizeof(int) * (4 * blk_.size() + 16));
        ev_.resize(2);
        for (auto &e : ev_) SDPG_CUDA(cudaEventCreate(&e));
    }

    int f1_chunk(const Blk &B) const {
        const size_t nn = (size_t)B.n * B.n;
        size_t c = (size_t)(1ull << 30) / (3 * nn * sizeof(V) + 1);
        if (c < 1) c = 1;
        if ((int)c > B.nF1) c = B.nF1 > 0 ? B.nF1 : 1;
        return (int)c;
    }

    static size_t gemm_bytes(int M, int Nn, int K, int batch) {
        GemmProblem<N> p{};
        p.M = M;
        p.Nn = Nn;
        p.K = K;
        p.batch = batch;
        p.A.sb = batch > 1 ? 1 : 0;
        p.B.sb = batch > 1 ? 1 : 0;
        return gemm_workspace_bytes<N>(p);
    }

    // ---------------------------------------------------------------- CUDA graphs
    //
    // A launch-heavy, host-sync-free sequence (a factorisation with its panel products)
    // runs eagerly on its first call (one-time set-up: tables, kernel attributes), is
    // captured into a graph on the second and replayed from then on: one host call
    // instead of hundreds, which is what bounds small problems and concurrent solvers.
    // Everything such a sequence touches (buffers, workspace offsets, sizes) is fixed
    // for the life of the solver.
    struct GraphSlot {
        cudaGraphExec_t exec = nullptr;
        int calls = 0;
        unsigned long long launches = 0;  // kernels in the graph (for the launch counter)
        GraphSlot() = default;
        GraphSlot(const GraphSlot &) = delete;
        GraphSlot(GraphSlot &&o) noexcept : exec(o.exec), calls(o.calls), launches(o.launches) { o.exec = nullptr; }
        ~GraphSlot() {
            if (exec) cudaGraphExecDestroy(exec);
        }
    };
    template <class F>
    void graphed(GraphSlot &g, cudaStream_t st, F &&f) {
        if (g_kt_on.load(std::memory_order_relaxed)) {  // per-kernel timing: plain launches
            f();
            return;
        }
        if (g.exec) {
            SDPG_CUDA(cudaGraphLaunch(g.exec, st));
            g_kernel_launches.fetch_add(g.launches, std::memory_order_relaxed);
            return;
        }
        if (g.calls++ == 0) {
            f();
            return;
        }
        cudaGraph_t graph = nullptr;
        const unsigned long long l0 = g_kernel_launches.load();
        SDPG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        capturing_ = true;
        try {
            f();
        } catch (...) {
            capturing_ = false;
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        capturing_ = false;
        SDPG_CUDA(cudaStreamEndCapture(st, &graph));
        g.launches = g_kernel_launches.load() - l0;
        const cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        SDPG_CUDA(e);
        SDPG_CUDA(cudaGraphLaunch(g.exec, st));
    }
    GraphSlot g_schur_chol_, g_schur_inv_;
    bool capturing_ = false;  // GEMMs issued into a graph are not bracketed by profiling events
    std::vector<GraphSlot> g_invchol_;  // per block: X (main stream), then Z (second stream)
    std::vector<GraphSlot> g_lanczos_;  // per block and side: every Lanczos step of a run

    // ---------------------------------------------------------------- memory helpers

    static constexpr int kSlots = 64;
    std::vector<void *> allocs_;
    void *dalloc_raw(size_t bytes) {
        void *p = nullptr;
        SDPG_CUDA(cudaMallocAsync(&p, bytes ? bytes : 16, st_));
        SDPG_CUDA(cudaMemsetAsync(p, 0, bytes ? bytes : 16, st_));
        allocs_.push_back(p);
        return p;
    }
    V *dalloc(size_t count) { return (V *)dalloc_raw(count * sizeof(V)); }
    template <class T>
    T *upload_new(const std::vector<T> &h) {
        h2d_ += (long long)(h.size() * sizeof(T));
        T *d = (T *)dalloc_raw(h.size() * sizeof(T));
        if (!h.empty()) {
            SDPG_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st_));
            SDPG_CUDA(cudaStreamSynchronize(st_));  // h is the caller's
        }
        return d;
    }
    void upload(V *d, const V *h, size_t count) {
        h2d_ += (long long)(count * sizeof(V));
        SDPG_CUDA(cudaMemcpyAsync(d, h, count * sizeof(V), cudaMemcpyHostToDevice, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
    }
    // read device scalar slots [0, cnt)
    std::vector<R> fetch(int cnt) {
        d2h_ += (long long)cnt * (long long)sizeof(V);
        std::vector<V> h(cnt);
        SDPG_CUDA(cudaMemcpyAsync(h.data(), slot_, cnt * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        std::vector<R> r(cnt);
        for (int i = 0; i < cnt; ++i) r[i] = R(h[i]);
        return r;
    }
    R fetch1(const V *d) {
        d2h_ += (long long)sizeof(V);
        V h;
        SDPG_CUDA(cudaMemcpyAsync(&h, d, sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        return R(h);
    }

    // ---------------------------------------------------------------- Lal-level helpers

    // C = alpha * op(A) * op(B) + beta * C on n x n blocks (Lal::multiply -> Rgemm)
    void mm(int n, V *C, const V *A, char ta, const V *Bm, char tb, const R &alpha = R(1), const R &beta = R(0)) {
        mm_on(st_, ws_, n, C, A, ta, Bm, tb, alpha, beta);
    }
    void mm_on(cudaStream_t st, Workspace &ws, int n, V *C, const V *A, char ta, const V *Bm, char tb,
               const R &alpha = R(1), const R &beta = R(0)) {
        GemmProblem<N> p{};
        p.M = n;
        p.Nn = n;
        p.K = n;
        p.batch = 1;
        p.A = operand_A<N>(ta, A, n, 0);
        p.B = operand_B<N>(tb, Bm, n, 0);
        p.C = C;
        p.ldc = n;
        p.sc = 0;
        p.alpha = alpha.v;
        p.beta = beta.v;
        gemm(p, st, ws);
    }
    void gemm(const GemmProblem<N> &p0) { gemm(p0, st_, ws_); }
    void gemm(const GemmProblem<N> &p0, cudaStream_t st, Workspace &ws) {
        GemmProblem<N> p = p0;
        if (prof_on_ && !capturing_) {
            if (prof_used_ * 2 + 2 > (int)prof_ev_.size()) {
                if (prof_used_ >= 4096) collect_gemm_events();
                while (prof_used_ * 2 + 2 > (int)prof_ev_.size()) {
                    cudaEvent_t e;
                    SDPG_CUDA(cudaEventCreate(&e));
                    prof_ev_.push_back(e);
                }
            }
            p.ev_before = prof_ev_[2 * prof_used_];
            p.ev_after = prof_ev_[2 * prof_used_ + 1];
            ++prof_used_;
            ++prof_launches_;
            prof_macs_ += (long long)p.M * p.Nn * p.K * p.batch;
        }
        const size_t mark = ws.used;
        ml_gemm<N>(p, ws, st);
        ws.used = mark;
        gemm_macs_ += (long long)p.M * p.Nn * p.K * p.batch;
    }
    // ret = sum over blocks of A_l . B_l  (Lal::let(ret,'=',A,'.',B) on DenseLinearSpace)
    R ip_blocks(V *Blk::*a, V *Blk::*b) {
        for (size_t l = 0; l < blk_.size(); ++l) {
            const size_t mark = ws_.used;
            k_dot<N>((long long)blk_[l].n * blk_[l].n, blk_[l].*a, blk_[l].*b, slot_ + l, ws_, st_);
            ws_.used = mark;
        }
        auto v = fetch((int)blk_.size());
        R s(0);
        for (auto &x : v) s += x;
        return s;
    }
    R ip_vec(const V *a, const V *b) {
        const size_t mark = ws_.used;
        k_dot<N>(m_, a, b, slot_, ws_, st_);
        ws_.used = mark;
        return fetch(1)[0];
    }
    // g = sum over blocks of A_i . M  (InputData::multi_InnerProductToA, sdpa_dataset.cpp:477-485)
    void multi_inner(V *Blk::*M, V *g) {
        SDPG_CUDA(cudaMemsetAsync(g, 0, m_ * sizeof(V), st_));
        for (auto &B : blk_) {
            const size_t mark = ws_.used;
            k_constraint_inner<N>(B.cons, B.*M, g, ws_, st_);
            ws_.used = mark;
        }
    }
    // M = sum_i A_i y_i  (InputData::multi_plusToA, sdpa_dataset.cpp:488-493)
    void multi_plus(const V *y, V *Blk::*M) {
        for (auto &B : blk_) k_constraint_plus<N>(B.cons, y, B.*M, st_);
    }
    void axpby_blocks(V *Blk::*out, const R &a, V *Blk::*x, const R &b, V *Blk::*y) {
        for (auto &B : blk_) k_axpby<N>((long long)B.n * B.n, a.v, B.*x, b.v, y ? B.*y : nullptr, B.*out, st_);
    }

    // ---------------------------------------------------------------- Newton (sdpa_newton.cpp)

    // Newton::compute_rMat, sdpa_newton.cpp:821-838
    void compute_rMat(bool corrector) {
        const R target = betaV_ * muCur_;
        axpby_blocks(&Blk::Rm, target, &Blk::Zinv, R(0), nullptr);
        axpby_blocks(&Blk::Rm, R(1), &Blk::Rm, R(-1), &Blk::X);
        if (corrector) {
            for (auto &B : blk_) {
                mm(B.n, B.W2, B.Dx, 'N', B.Dz, 'N');
                mm(B.n, B.W1, B.W2, 'N', B.Zinv, 'N');
            }
            axpby_blocks(&Blk::Rm, R(1), &Blk::Rm, R(-1), &Blk::W1);
        }
    }

    // Newton::Make_gVec, sdpa_newton.cpp:840-895
    void Make_gVec(bool corrector, bool keep_rmat = false) {
        if (!keep_rmat) compute_rMat(corrector);
        if (phase_ == pFEAS || phase_ == noINFO) {
            if (!corrector) {
                for (auto &B : blk_) {
                    mm(B.n, B.W2, B.X, 'N', B.Dres, 'N');
                    mm(B.n, B.XRDZ, B.W2, 'N', B.Zinv, 'N');
                }
            }
            axpby_blocks(&Blk::W1, R(1), &Blk::Rm, R(-1), &Blk::XRDZ);
        } else {
            for (auto &B : blk_) k_copy<N>((long long)B.n * B.n, B.Rm, B.W1, st_);
        }
        multi_inner(&Blk::W1, g_);
        k_axpby<N>(m_, R(-1).v, g_, R(1).v, p_, g_, st_);  // g = -g + p
    }

    // Newton::compute_bMat_dense_SDP, sdpa_newton.cpp:1007-1096 (via Make_bMat :1251-1272)
    void Make_bMat() {
        SDPG_CUDA(cudaMemsetAsync(B_, 0, (size_t)m_ * m_ * sizeof(V), st_));
        for (auto &B : blk_) {
            k_schur_f3<N>(B.cons, B.X, B.Zinv, B_, m_, st_);
            if (B.nF1 == 0) continue;
            const int n = B.n;
            const long long nn = (long long)n * n;
            const int chunk = f1_chunk(B);
            for (int c0 = 0; c0 < B.nF1; c0 += chunk) {
                const int cnt = std::min(chunk, B.nF1 - c0);
                const size_t mark = ws_.used;
                V *Ad = (V *)ws_.carve((size_t)cnt * nn * sizeof(V));
                V *T = (V *)ws_.carve((size_t)cnt * nn * sizeof(V));
                const int *owners = B.f1_owners + c0;
                k_densify<N>(B.cons, owners, cnt, Ad, st_);
                // T_t = A_t Zinv ; G_t = X T_t   (F1: work1 = A_i*invZ, work2 = X*work1)
                GemmProblem<N> p{};
                p.M = n;
                p.Nn = n;
                p.K = n;
                p.batch = cnt;
                p.A = operand_A<N>('N', Ad, n, nn);
                p.B = operand_B<N>('N', B.Zinv, n, 0);
                p.C = T;
                p.ldc = n;
                p.sc = nn;
                p.alpha = R(1).v;
                p.beta = R(0).v;
                gemm(p);
                p.A = operand_A<N>('N', B.X, n, 0);
                p.B = operand_B<N>('N', T, n, nn);
                p.C = Ad;  // G overwrites the densified constraints
                gemm(p);
                V *G = Ad;
                k_schur_f1_sparse<N>(B.cons, owners, cnt, G, B_, m_, st_);
                const int nd = B.cons.ndense;
                if (nd > 0) {
                    V *P = (V *)ws_.carve((size_t)cnt * nd * sizeof(V));
                    if ((long long)cnt * nd >= 1024) {
                        GemmProblem<N> q{};
                        q.M = cnt;
                        q.Nn = nd;
                        q.K = (int)nn;
                        q.batch = 1;
                        q.A = operand_A<N>('T', G, nn, 0);
                        q.B = operand_B<N>('N', B.cons.dense, nn, 0);
                        q.C = P;
                        q.ldc = cnt;
                        q.sc = 0;
                        q.alpha = R(1).v;
                        q.beta = R(0).v;
                        gemm(q);
                    } else {
                        std::vector<long long> xo((size_t)cnt * nd), yo((size_t)cnt * nd);
                        for (int d = 0; d < nd; ++d)
                            for (int t = 0; t < cnt; ++t) {
                                xo[t + (size_t)cnt * d] = (long long)t * nn;
                                yo[t + (size_t)cnt * d] = (long long)d * nn;
                            }
                        long long *dxo = (long long *)ws_.carve(xo.size() * sizeof(long long));
                        long long *dyo = (long long *)ws_.carve(yo.size() * sizeof(long long));
                        h2d_ += (long long)xo.size() * 16;
                        SDPG_CUDA(cudaMemcpyAsync(dxo, xo.data(), xo.size() * 8, cudaMemcpyHostToDevice, st_));
                        SDPG_CUDA(cudaMemcpyAsync(dyo, yo.data(), yo.size() * 8, cudaMemcpyHostToDevice, st_));
                        k_dot_batched<N>(nn, G, dxo, B.cons.dense, dyo, cnt * nd, P, ws_, st_);
                        SDPG_CUDA(cudaStreamSynchronize(st_));  // host offset arrays go out of scope
                    }
                    k_schur_f1_dense_scatter<N>(B.cons, owners, cnt, P, B_, m_, st_);
                }
                ws_.used = mark;
            }
        }
    }

    // Newton::compute_DyVec, sdpa_newton.cpp:1308-1344 (Lal::choleskyFactorWithAdjust + solveSystems)
    bool compute_DyVec(bool corrector) {
        if (!corrector) {
            graphed(g_schur_chol_, st_, [&] { ml_potrf<N>(m_, B_, m_, info_, ws_, st_); });
            int info = 0;
            d2h_ += (long long)sizeof(int);
            SDPG_CUDA(cudaMemcpyAsync(&info, info_, sizeof(int), cudaMemcpyDeviceToHost, st_));
            SDPG_CUDA(cudaStreamSynchronize(st_));
            if (info != 0) return false;
            // L^{-1} once per factorisation (recursive, GEMM based); each solve is then
            // two triangular matrix-vector products, read column-wise for coalescing
            graphed(g_schur_inv_, st_, [&] {
                ml_trtri_lower<N>(m_, B_, m_, BLinv_, ws_, st_);
                k_transpose<N>(m_, BLinv_, BLinvT_, st_);
            });
        }
        k_matvec<N>(m_, BLinvT_, 'T', 2, g_, Dytmp_, st_);  // L^{-1} g
        k_matvec<N>(m_, BLinv_, 'T', 1, Dytmp_, Dy_, st_);  // L^{-T} L^{-1} g
        return true;
    }

    // Newton::compute_DzMat, sdpa_newton.cpp:1346-1356
    void compute_DzMat() {
        multi_plus(Dy_, &Blk::Dz);
        if (phase_ == pFEAS || phase_ == noINFO) axpby_blocks(&Blk::Dz, R(-1), &Blk::Dz, R(1), &Blk::Dres);
        else axpby_blocks(&Blk::Dz, R(-1), &Blk::Dz, R(0), nullptr);
    }

    // Newton::compute_DxMat, sdpa_newton.cpp:1358-1373
    void compute_DxMat() {
        for (auto &B : blk_) {
            mm(B.n, B.W2, B.X, 'N', B.Dz, 'N');
            mm(B.n, B.W1, B.W2, 'N', B.Zinv, 'N');
        }
        axpby_blocks(&Blk::Dx, R(1), &Blk::Rm, R(-1), &Blk::W1);
        for (auto &B : blk_) k_symmetrize<N>(B.n, B.Dx, st_);
    }

    // The corrector again with beta + delta: R Z^-1 is affine in beta (compute_rMat), so
    // it is shifted by delta mu Z^-1 and the rest of the direction recomputed from it.
    void newton_rebeta(const R &delta) {
        axpby_blocks(&Blk::Rm, R(1), &Blk::Rm, delta * muCur_, &Blk::Zinv);
        Make_gVec(true, true);
        compute_DyVec(true);
        compute_DzMat();
        compute_DxMat();
    }

    // Newton::Mehrotra, sdpa_newton.cpp:1375-1414
    bool newton(int corrector) override {
        ev_start();
        Make_gVec(corrector);
        tm_.rmat_gvec += ev_stop();
        if (!corrector) {
            ev_start();
            Make_bMat();
            tm_.schur += ev_stop();
        }
        ev_start();
        const bool ok = compute_DyVec(corrector);
        tm_.cholesky += ev_stop();
        if (!ok) return false;
        ev_start();
        compute_DzMat();
        compute_DxMat();
        tm_.dxdz += ev_stop();
        return true;
    }

    // ---------------------------------------------------------------- eigenvalues (sdpa_jordan.cpp, sdpa_linear.cpp)

    // One Lanczos run (Lal::getMinEigen, sdpa_linear.cpp:27-124) on L Xm L^T for one block
    // and side.  The steps and the loop test run on the device (k_lanczos_step); the host
    // enqueues every step the run can take and reads the result once.
    struct Lz {
        Blk *B;
        int side, n, kgo;
        V *L, *Xm, *Lt;
        cudaStream_t st;
        Workspace *ws;
        V *hp;  // 16 pinned slots: the run's state slots, flags at 12
        R min, error, beta;
        std::vector<int> eig;  // steps with a tridiagonal eigenvalue solve
        bool active;
    };

    // all runs at once: one host synchronisation for all of them
    void lanczos_all(std::vector<Lz> &T) {
        if (16 * T.size() > (size_t)kPinned - 8) throw sdpg_error(SDPG_ERR_TOO_LARGE, "too many Lanczos runs at once");
        for (size_t i = 0; i < T.size(); ++i) {
            Lz &t = T[i];
            Blk &B = *t.B;
            const int s = t.side;
            t.hp = pinned_ + 16 * i;
            // the Lanczos operator L X L^T, formed once per run (symmetric up to rounding;
            // its columns are read as rows)
            mm_on(t.st, *t.ws, t.n, B.Mtmp[s], t.Xm, 'N', t.L, 'T');
            mm_on(t.st, *t.ws, t.n, B.Mop[s], t.L, 'N', B.Mtmp[s], 'N');
            k_fill<N>(t.n, B.r[s], ml_one<N>(), t.st);
            SDPG_CUDA(cudaMemsetAsync(B.q[s], 0, t.n * sizeof(V), t.st));
            // the loop's initial state (sdpa_linear.cpp:33-56): r = 1, beta = |r|,
            // min = 1e51, min_old = 1e52, error = 1e10
            const R beta = rsqrt_(R(t.n));
            const R sq_n = beta, sq_n9 = rsqrt_(R(t.n) + R(9));
            for (int q = 0; q < 12; ++q) t.hp[q] = ml_zero<N>();
            t.hp[0] = (R(1) / beta).v;
            t.hp[1] = beta.v;
            t.hp[8] = R(1.0e+51).v;
            t.hp[9] = R(1.0e+52).v;
            t.hp[10] = R(1.0e+10).v;
            int *flags = reinterpret_cast<int *>(t.hp + 12);
            flags[0] = 1;
            flags[1] = 0;
            h2d_ += 12 * (long long)sizeof(V) + 2 * (long long)sizeof(int);
            SDPG_CUDA(cudaMemcpyAsync(B.sl[s], t.hp, 12 * sizeof(V), cudaMemcpyHostToDevice, t.st));
            SDPG_CUDA(cudaMemcpyAsync(B.lzctl[s], flags, 2 * sizeof(int), cudaMemcpyHostToDevice, t.st));
            // the loop bound k < sqrt(n) + 10 as a step count, and the static schedule of
            // the eigenvalue solves (kk >= sqrt(k) || k == n - 1 || k > sqrt(n + 9))
            t.kgo = 0;
            while (R(t.kgo) < sq_n + R(10)) ++t.kgo;
            const int kmax = B.lanczos_kmax;
            t.eig.assign(kmax + 1, 0);
            int kk = 0;
            for (int k = 0; k <= kmax; ++k, ++kk) {
                t.eig[k] = (R(kk) >= rsqrt_(R(k)) || k == t.n - 1 || R(k) > sq_n9) ? 1 : 0;
                if (t.eig[k]) kk = 0;
            }
            t.active = t.n > 0 && kmax > 1;
            t.ws->ensure_side();  // the eigenvalue steps' tridiagonal solves run there
        }
        // (the pinned slots are next written by stream-ordered copies, after the uploads)
        lanczos_graphed(T);
        for (Lz &t : T) {
            d2h_ += 11 * (long long)sizeof(V);
            SDPG_CUDA(cudaMemcpyAsync(t.hp, t.B->sl[t.side], 11 * sizeof(V), cudaMemcpyDeviceToHost, t.st));
        }
        SDPG_CUDA(cudaStreamSynchronize(st_));
        SDPG_CUDA(cudaStreamSynchronize(st2_));
        for (Lz &t : T) {
            t.beta = R(t.hp[1]);
            t.min = R(t.hp[8]);
            t.error = R(t.hp[10]);
        }
    }

    // Every step a run can take, enqueued at once as one CUDA graph per (block, side)
    // (captured on the second call, replayed after): the steps past the loop's end return
    // at once on the device flag, and the host waits only for the final result.
    void lanczos_graphed(std::vector<Lz> &T) {
        if (g_lanczos_.size() != 2 * blk_.size()) g_lanczos_.resize(2 * blk_.size());
        for (Lz &t : T) {
            if (!t.active) continue;
            Blk &B = *t.B;
            const int s = t.side;
            const size_t slot = 2 * (size_t)(t.B - blk_.data()) + (size_t)s;
            graphed(g_lanczos_[slot], t.st, [&] {
                for (int k = 0; k < t.n && k + 1 < B.lanczos_kmax; ++k)
                    k_lanczos_step<N>(t.n, B.Mop[s], B.r[s], B.q[s], B.qold[s], B.w[s], B.td[s], B.te[s], B.sl[s],
                                      B.lzctl[s], status_, k, t.eig[k], t.kgo, B.lanczos_kmax, t.st, t.ws->side,
                                      t.ws->ev[0], t.ws->ev[1]);
            });
        }
    }

    // Lal::getMinEigenValue on L*X*L^T for blocks of size <= 20 (sdpa_jordan.cpp:63-68):
    // enqueue only; the value lands in B.sl[side][4]
    void small_min_issue(Blk &B, int side, V *L, V *Xm, cudaStream_t st, Workspace &ws) {
        const int n = B.n;
        V *w1 = side == 0 ? B.W1 : B.SW1;
        V *w2 = side == 0 ? B.W2 : B.SW2;
        mm_on(st, ws, n, w2, Xm, 'N', L, 'T');
        mm_on(st, ws, n, w1, L, 'N', w2, 'N');
        k_tridiagonalize_small<N>(n, w1, B.td[side], B.te[side], st);
        k_tridiag_min<N>(n, B.td[side], B.te[side], B.sl[side] + 4, status_, st);
    }

    // Jal::getMinEigen(L_X^-1, dX) and Jal::getMinEigen(L_Z^-1, dZ) (sdpa_jordan.cpp:55-88),
    // both sides and all blocks at once: the X side on the main stream, the Z side on the
    // second stream.
    void min_eigen_both(R *minX, R *minZ) {
        // the Z side reads dZ / L_Z^-1 written on the main stream
        SDPG_CUDA(cudaEventRecord(ev_fork_, st_));
        SDPG_CUDA(cudaStreamWaitEvent(st2_, ev_fork_, 0));
        std::vector<Lz> T;
        for (auto &B : blk_) {
            for (int side = 0; side < 2; ++side) {
                V *L = side == 0 ? B.LX : B.LZ;
                V *Xm = side == 0 ? B.Dx : B.Dz;
                cudaStream_t st = side == 0 ? st_ : st2_;
                Workspace &ws = side == 0 ? ws_ : ws2_;
                if (B.lp) {
                    k_lp_ratio_min<N>(B.n, Xm, L, B.sl[side] + 4, st);
                } else if (B.n > 20) {
                    Lz t{};
                    t.B = &B;
                    t.side = side;
                    t.n = B.n;
                    t.L = L;
                    t.Xm = Xm;
                    t.Lt = side == 0 ? B.Lt : B.F;
                    t.st = st;
                    t.ws = &ws;
                    T.push_back(t);
                } else {
                    small_min_issue(B, side, L, Xm, st, ws);
                }
            }
        }
        lanczos_all(T);
        *minX = R(1.0E50);
        *minZ = R(1.0E50);
        // small-block results
        std::vector<V> h(2 * blk_.size());
        for (size_t l = 0; l < blk_.size(); ++l)
            if (blk_[l].n <= 20 || blk_[l].lp)
                for (int side = 0; side < 2; ++side) {
                    d2h_ += (long long)sizeof(V);
                    SDPG_CUDA(cudaMemcpyAsync(&h[2 * l + side], blk_[l].sl[side] + 4, sizeof(V),
                                              cudaMemcpyDeviceToHost, st_));
                }
        SDPG_CUDA(cudaStreamSynchronize(st_));
        size_t ti = 0;
        for (size_t l = 0; l < blk_.size(); ++l) {
            for (int side = 0; side < 2; ++side) {
                R v;
                if (blk_[l].n > 20 && !blk_[l].lp) {
                    const Lz &t = T[ti++];
                    v = t.min - rabs(t.error * t.beta);
                } else {
                    v = R(h[2 * l + side]);
                }
                R &target = side == 0 ? *minX : *minZ;
                if (v < target) target = v;
            }
        }
    }

    R getMinEigen(V *Blk::*L, V *Blk::*Xm) {
        R mx, mz;
        min_eigen_both(&mx, &mz);
        return (L == &Blk::LX) ? mx : mz;
    }

    // ---------------------------------------------------------------- step length (sdpa_parts.cpp)

    // StepLength::computeStepLength, sdpa_parts.cpp:298-360
    void computeStepLength() {
        const R alphaBD(100.0);
        R minX, minZ;
        min_eigen_both(&minX, &minZ);
        if (-minX > R(1.0) / alphaBD) aP_ = -R(1.0) / minX;
        else aP_ = alphaBD;
        if (-minZ > R(1.0) / alphaBD) aD_ = -R(1.0) / minZ;
        else aD_ = alphaBD;
    }

    // StepLength::MehrotraPredictor (:362-410) / MehrotraCorrector (:412-523)
    void step_length(int corrector) override {
        ev_start();
        if (!corrector) {
            aP_ = aD_ = R(0.9);
        } else {
            computeStepLength();
            aP_ = R(par_.gammaStar) * aP_;
            aD_ = R(par_.gammaStar) * aD_;
        }
        if (phase_ == noINFO || phase_ == dFEAS) {
            if (aP_ > R(1.0)) aP_ = R(1.0);
        } else {
            const R incPrimalObj = ip_blocks(&Blk::C, &Blk::Dx);
            if (incPrimalObj > R(0.0)) {
                if (aP_ > aD_) aP_ = aD_;
                if (aP_ > R(1.0)) aP_ = R(1.0);
            }
        }
        if (phase_ == noINFO || phase_ == pFEAS) {
            if (aD_ > R(1.0)) aD_ = R(1.0);
        } else {
            const R incDualObj = ip_vec(b_, Dy_);
            if (incDualObj < R(0.0)) {
                if (aD_ > aP_) aD_ = aP_;
                if (aD_ > R(1.0)) aD_ = R(1.0);
            }
        }
        if (corrector) {
            const R xi(3.0);
            if (reductionOn_ && (phase_ == noINFO || phase_ == pFEAS || phase_ == dFEAS)) {
                const R xMatvMat = ip_blocks(&Blk::X, &Blk::Dz);
                const R uMatzMat = ip_blocks(&Blk::Dx, &Blk::Z);
                const R uMatvMat = ip_blocks(&Blk::Dx, &Blk::Dz);
                R thetaMax = rmax((R(1.0) - aP_) * thP_, (R(1.0) - aD_) * thD_);
                R muNew = muCur_ + (aP_ * uMatzMat + aD_ * xMatvMat + aP_ * aD_ * uMatvMat) / R(nDim_);
                while (thetaMax * thetaMax * muInit_ > xi * muNew) {
                    const R alphaMax = R(0.95) * rmax(aP_, aD_);
                    aP_ = rmin(aP_, alphaMax);
                    aD_ = rmin(aD_, alphaMax);
                    thetaMax = rmax((R(1.0) - aP_) * thP_, (R(1.0) - aD_) * thD_);
                    muNew = muCur_ + (aP_ * uMatzMat + aD_ * xMatvMat + aP_ * aD_ * uMatvMat) / R(nDim_);
                    if (aP_ < R(1.0e-6) && aD_ < R(1.0e-6)) break;
                }
            }
            if (phase_ == pdFEAS) {
                const R objValDual = ip_vec(b_, y_);
                const R objValPrimal = ip_blocks(&Blk::C, &Blk::X);
                R incDualObj = ip_vec(b_, Dy_);
                incDualObj *= aD_;
                R incPrimalObj = ip_blocks(&Blk::C, &Blk::Dx);
                incPrimalObj *= aP_;
                const R maxRatio = (objValDual - objValPrimal) / (incPrimalObj - incDualObj);
                if (maxRatio > R(0.0) && maxRatio < R(1.0)) {
                    aP_ *= maxRatio;
                    aD_ *= maxRatio;
                }
            }
        }
        tm_.steplen += ev_stop();
    }

    // DirectionParameter::MehrotraPredictor (:543-553) and Switch::MehrotraPredictor (:605-612)
    void direction_predictor() {
        reductionOn_ = (phase_ == noINFO || phase_ == pFEAS || phase_ == dFEAS) ? 1 : 0;
        const R nu(2.0);
        if (phase_ == pdFEAS) betaV_ = R(0.0);
        else {
            betaV_ = R(par_.betaBar);
            if (!reductionOn_) betaV_ = nu;
        }
    }

    // DirectionParameter::MehrotraCorrector, sdpa_parts.cpp:555-586
    void direction_corrector() {
        const R xMatvMat = ip_blocks(&Blk::X, &Blk::Dz);
        const R uMatzMat = ip_blocks(&Blk::Dx, &Blk::Z);
        const R uMatvMat = ip_blocks(&Blk::Dx, &Blk::Dz);
        const R muTarget = muCur_ + (aP_ * uMatzMat + aD_ * xMatvMat + aP_ * aD_ * uMatvMat) / R(nDim_);
        betaV_ = muTarget / muCur_;
        if (betaV_ < R(1.0)) betaV_ = betaV_ * betaV_;
        if (phase_ == pdFEAS) {
            if (betaV_ < R(par_.betaStar)) betaV_ = R(par_.betaStar);
            if (betaV_ > R(1.0)) betaV_ = R(1.0);
        } else {
            if (betaV_ < R(par_.betaBar)) betaV_ = R(par_.betaBar);
        }
    }

    // ---------------------------------------------------------------- iterate update (sdpa_dataset.cpp)

    // Jal::getInvChol / getInvCholAndInv (sdpa_jordan.cpp:123-171) for one block, enqueued
    // on `st`: factor a copy of A (Lal::getCholesky), invert the factor, optionally form
    // Inv = Linv^T Linv (Rtrmm).  A failed factorisation leaves its column in *info.
    void inv_chol_issue(Blk &B, V *A, V *Fbuf, V *Linv, V *Inv, int *info, cudaStream_t st, Workspace &ws) {
        const int n = B.n;
        k_copy<N>((long long)n * n, A, Fbuf, st);
        ml_potrf<N>(n, Fbuf, n, info, ws, st);
        k_zero_strict_upper<N>(n, Fbuf, st);
        ml_trtri_lower<N>(n, Fbuf, n, Linv, ws, st);
        if (Inv) mm_on(st, ws, n, Inv, Linv, 'T', Linv, 'N');
    }

    // Solutions::computeInverse, sdpa_dataset.cpp:96-118: the X and Z chains are
    // independent and run concurrently (X on the main stream, Z on the second stream).
    bool computeInverse() {
        const size_t nb = blk_.size();
        SDPG_CUDA(cudaEventRecord(ev_fork_, st_));
        SDPG_CUDA(cudaStreamWaitEvent(st2_, ev_fork_, 0));
        if (g_invchol_.size() != 2 * nb) g_invchol_.resize(2 * nb);
        for (size_t l = 0; l < nb; ++l)
            graphed(g_invchol_[l], st_, [&] {
                inv_chol_issue(blk_[l], blk_[l].X, blk_[l].F, blk_[l].LX, nullptr, info_all_ + l, st_, ws_);
            });
        for (size_t l = 0; l < nb; ++l)
            graphed(g_invchol_[nb + l], st2_, [&] {
                inv_chol_issue(blk_[l], blk_[l].Z, blk_[l].W2, blk_[l].LZ, blk_[l].Zinv, info_all_ + nb + l, st2_,
                               ws2_);
            });
        SDPG_CUDA(cudaEventRecord(ev_join_, st2_));
        SDPG_CUDA(cudaStreamWaitEvent(st_, ev_join_, 0));
        std::vector<int> info(2 * nb);
        d2h_ += (long long)(2 * nb * sizeof(int));
        SDPG_CUDA(cudaMemcpyAsync(info.data(), info_all_, 2 * nb * sizeof(int), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        for (int v : info)
            if (v != 0) return false;
        return true;
    }

    // Solutions::update, sdpa_dataset.cpp:120-143
    bool update() override {
        ev_start();
        axpby_blocks(&Blk::X, R(1), &Blk::X, aP_, &Blk::Dx);
        k_axpby<N>(m_, R(1).v, y_, aD_.v, Dy_, y_, st_);
        axpby_blocks(&Blk::Z, R(1), &Blk::Z, aD_, &Blk::Dz);
        const R cannot_move(1.0e-4);
        if (aP_ < cannot_move && aD_ < cannot_move) {
            tm_.update += ev_stop();
            return false;
        }
        const bool ok = computeInverse();
        tm_.update += ev_stop();
        return ok;
    }

    // ---------------------------------------------------------------- residuals and control

    // Residuals::compute, sdpa_dataset.cpp:625-646
    void residuals() override {
        ev_start();
        multi_inner(&Blk::X, p_);
        k_axpby<N>(m_, R(-1).v, p_, R(1).v, b_, p_, st_);
        multi_plus(y_, &Blk::Dres);
        axpby_blocks(&Blk::Dres, R(-1), &Blk::Dres, R(1), &Blk::C);
        axpby_blocks(&Blk::Dres, R(1), &Blk::Dres, R(-1), &Blk::Z);
        {
            const size_t mark = ws_.used;
            k_maxabs<N>(m_, p_, slot_, ws_, st_);
            for (size_t l = 0; l < blk_.size(); ++l)
                k_maxabs<N>((long long)blk_[l].n * blk_[l].n, blk_[l].Dres, slot_ + 1 + l, ws_, st_);
            ws_.used = mark;
        }
        auto v = fetch(1 + (int)blk_.size());
        normP_ = v[0];
        normD_ = R(0.0);
        for (size_t l = 0; l < blk_.size(); ++l)
            if (v[1 + l] > normD_) normD_ = v[1 + l];
        tm_.residual += ev_stop();
    }

    // Phase::updateCheck, sdpa_parts.cpp:932-1011 (REVERSE_PRIMAL_DUAL bounds)
    bool phase_updateCheck() {
        const R NONZERO(1.0e-6);
        const R accuracy(par_.epsilonDash);
        phase_ = noINFO;
        if (normP_ <= accuracy) phase_ = (normD_ <= accuracy) ? pdFEAS : pFEAS;
        if (phase_ == noINFO && normD_ <= accuracy) phase_ = dFEAS;
        if (phase_ == pdFEAS) {
            const R mean = (rabs(objP_) + rabs(objD_)) / R(2.0);
            const R PDgap = rabs(objP_ - objD_);
            const R dominator = (mean < R(1.0)) ? R(1.0) : mean;
            if (PDgap / dominator <= R(par_.epsilonStar)) {
                phase_ = pdOPT;
                return false;
            }
        }
        if (phase_ == noINFO && rho_ > R(1.0) + NONZERO) {
            phase_ = pdINF;
            return false;
        }
        if (phase_ == pFEAS) {
            if (objP_ <= -R(par_.upperBound)) {
                phase_ = pUNBD;
                return false;
            }
            if (rho_ > R(1.0) + NONZERO) {
                phase_ = pFEAS_dINF;
                return false;
            }
        }
        if (phase_ == dFEAS) {
            if (objD_ >= -R(par_.lowerBound)) {
                phase_ = dUNBD;
                return false;
            }
            if (rho_ > R(1.0) + NONZERO) {
                phase_ = pINF_dFEAS;
                return false;
            }
        }
        return true;
    }

    // SolveInfo::update(lambda, ...), sdpa_parts.cpp:798-860
    void solveInfo_update() {
        objP_ = ip_blocks(&Blk::C, &Blk::X);
        objD_ = ip_vec(b_, y_);
        const R primal = thP_, dual = thD_, omega(par_.omegaStar);
        rho_ = R(0.0);
        const R x0z0 = R(nDim_) * muInit_;
        const R xMatzMat = R(nDim_) * muCur_;
        R x0zMat(0.0), xMatz0(0.0);
        const R lambda(par_.lambdaStar);
        for (size_t l = 0; l < blk_.size(); ++l) {
            k_trace<N>(blk_[l].n, blk_[l].Z, slot_ + 2 * l, st_);
            k_trace<N>(blk_[l].n, blk_[l].X, slot_ + 2 * l + 1, st_);
        }
        auto tr = fetch(2 * (int)blk_.size());
        // the reference accumulates lambda * Z_ii element by element; the sum of the
        // traces times lambda agrees to the working precision
        for (size_t l = 0; l < blk_.size(); ++l) {
            x0zMat += lambda * tr[2 * l];
            xMatz0 += lambda * tr[2 * l + 1];
        }
        const R accuracy(par_.epsilonDash);
        if (normP_ <= accuracy && xMatz0 < etaP_) etaP_ = xMatz0;
        if (normD_ <= accuracy && x0zMat < etaD_) etaD_ = x0zMat;
        if (normP_ > accuracy && normD_ <= accuracy)
            rho_ = primal * x0zMat / ((primal + (R(1.0) - primal) * omega) * etaD_ + xMatzMat);
        if (normP_ <= accuracy && normD_ > accuracy)
            rho_ = dual * xMatz0 / ((dual + (R(1.0) - dual) * omega) * etaP_ + xMatzMat);
        if (normP_ > accuracy && normD_ > accuracy)
            rho_ = (dual * xMatz0 + primal * x0zMat) /
                   ((primal * dual + omega * (primal * (R(1.0) - dual) + (R(1.0) - primal) * dual)) * x0z0 + xMatzMat);
    }

    // Solutions::initialize (sdpa_dataset.cpp:35-60) and the set-up part of pinpal
    // (sdpa_main.cpp:229-287); with a policy attached (flag 2) the point is set up once at
    // param.sdpa's lambdaStar, the policy reads it and proposes the lambdaStar used instead
    void initialize() override {
        par_.lambdaStar = lambda_default_;
        pol_lambda_prop_ = 0;
        pol_props_ = pol_fallbacks_ = 0;
        init_point();
        lastAP_ = lastAD_ = R(0.0);
        feats_.clear();
        feats_.push_back(policy_features(betaV_));
        if (policy_ && (pol_flags_ & 2)) {
            float y[kPolOut];
            policy_eval(feats_[0], y);
            const double e = std::min(6.0, std::max(-3.0, (double)y[0]));
            pol_lambda_prop_ = pow(10.0, e);
            par_.lambdaStar = pol_lambda_prop_;
            init_point();
        }
    }

    std::vector<int> block_structure() const override {
        std::vector<int> bs;
        for (const Blk &B : blk_) bs.push_back(B.lp ? -B.n : B.n);
        return bs;
    }
    void set_initial_point(const InitPoint &ip) override {
        if ((int)ip.x0.size() != m_) throw sdpg_error(SDPG_ERR_ARG, "initial point: x0 has the wrong length");
        for (const InitEntry &e : ip.entries)
            if (e.block < 0 || e.block >= (int)blk_.size() || e.i < 0 || e.j < 0 || e.i >= blk_[e.block].n ||
                e.j >= blk_[e.block].n || (e.target != 1 && e.target != 2))
                throw sdpg_error(SDPG_ERR_ARG, "initial point: entry out of range");
        init_ = ip;
        has_init_ = true;
        initialized_ = false;
    }

    void init_point() {
        const R lambda(par_.lambdaStar);
        const R invsq = R(1.0) / rsqrt_(lambda);
        const R inv = R(1.0) / lambda;
        for (auto &B : blk_) {
            k_set_identity<N>(B.n, B.X, lambda.v, st_);
            k_set_identity<N>(B.n, B.Z, lambda.v, st_);
            k_set_identity<N>(B.n, B.LX, invsq.v, st_);
            k_set_identity<N>(B.n, B.LZ, invsq.v, st_);
            k_set_identity<N>(B.n, B.Zinv, inv.v, st_);
        }
        SDPG_CUDA(cudaMemsetAsync(y_, 0, m_ * sizeof(V), st_));
        if (has_init_) {
            // main, sdpa_main.cpp:237-251: the file's entries over lambdaStar * I (both
            // triangles, DenseLinearSpace::setElement_SDP), y = -x0, then the inverses
            for (size_t l = 0; l < blk_.size(); ++l) {
                Blk &B = blk_[l];
                const size_t nn = (size_t)B.n * B.n;
                std::vector<V> Xh(nn, ml_zero<N>()), Zh(nn, ml_zero<N>());
                for (int k = 0; k < B.n; ++k) Xh[k + (size_t)B.n * k] = Zh[k + (size_t)B.n * k] = lambda.v;
                for (const InitEntry &e : init_.entries) {
                    if (e.block != (int)l) continue;
                    std::vector<V> &M = e.target == 1 ? Zh : Xh;
                    M[e.i + (size_t)B.n * e.j] = M[e.j + (size_t)B.n * e.i] = narrow<N>(e.v);
                }
                upload(B.X, Xh.data(), nn);
                upload(B.Z, Zh.data(), nn);
            }
            std::vector<V> yh(m_);
            for (int k = 0; k < m_; ++k) yh[k] = ml_neg(narrow<N>(init_.x0[k]));
            upload(y_, yh.data(), m_);
            if (!computeInverse())
                throw sdpg_error(SDPG_ERR_NOT_PD, "initial point: a matrix is not positive definite");
        }
        residuals();
        initNormP_ = normP_;
        initNormD_ = normD_;
        aP_ = aD_ = R(0.0);
        betaV_ = R(par_.betaStar);
        reductionOn_ = 1;
        // AverageComplementarity::initialize (sdpa_parts.cpp:633-643)
        muInit_ = has_init_ ? ip_blocks(&Blk::X, &Blk::Z) / R(nDim_) : lambda * lambda;
        muCur_ = muInit_;
        const R accuracy(par_.epsilonDash);
        thP_ = (initNormP_ < accuracy) ? R(0.0) : R(1.0);
        thD_ = (initNormD_ < accuracy) ? R(0.0) : R(1.0);
        rho_ = R(1.0);
        etaP_ = R(par_.omegaStar) * R(nDim_) * muInit_;
        etaD_ = etaP_;
        objP_ = ip_blocks(&Blk::C, &Blk::X);
        objD_ = ip_vec(b_, y_);
        phase_updateCheck();
        iter_ = 0;
        hist_.clear();
        printed_.clear();
        initialized_ = true;
        stopped_ = false;
        cannot_move_ = false;
    }

    void record_iteration() {
        IterRecord r;
        r.it = iter_;
        r.mu = muCur_.d();
        r.thetaP = thD_.d();  // printed with REVERSE_PRIMAL_DUAL (sdpa_io.cpp:764-796)
        r.thetaD = thP_.d();
        r.objP = (-objD_).d();
        r.objD = (-objP_).d();
        r.alphaP = aD_.d();
        r.alphaD = aP_.d();
        r.beta = betaV_.d();
        hist_.push_back(r);
    }

    // IO::printOneIteration (REVERSE_PRIMAL_DUAL branch), sdpa_io.cpp:764-796
    std::string iteration_line() const {
        char buf[512];
        snprintf(buf, sizeof buf, "%2d %s %s %s %s %s %s %s %s\n", iter_, muCur_.fmt(1).c_str(), thD_.fmt(1).c_str(),
                 thP_.fmt(1).c_str(), (-objD_).fmt(2, true).c_str(), (-objP_).fmt(2, true).c_str(),
                 aD_.fmt(1).c_str(), aP_.fmt(1).c_str(), betaV_.fmt(2).c_str());
        return buf;
    }
    void print_iteration(FILE *f) {
        const std::string line = iteration_line();
        if (printed_.size() < hist_.size()) printed_.push_back(line);
        if (!f) return;
        fputs(line.c_str(), f);
        fflush(f);
    }

    void trace_line() {
        if (!trace_) return;
        fprintf(trace_, "it=%d mu=%s objP=%s objD=%s aP=%s aD=%s beta=%s\n", iter_, muCur_.fmt(30).c_str(),
                objP_.fmt(30).c_str(), objD_.fmt(30).c_str(), aP_.fmt(30).c_str(), aD_.fmt(30).c_str(),
                betaV_.fmt(30).c_str());
        fflush(trace_);
    }

    // SDPG_ERR_TIMEOUT if a tensor-core GEMM or a Cholesky panel of this solver gave up a
    // bounded wait (its results, and everything computed from them, are then invalid)
    void check_tensor_timeout() {
        if (!tc_error_) return;
        int st = 0;
        d2h_ += (long long)sizeof(int);
        SDPG_CUDA(cudaMemcpyAsync(&st, tc_error_, sizeof(int), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        if (st != 0) throw sdpg_error(SDPG_ERR_TIMEOUT, "tensor-core GEMM or Cholesky panel: a bounded wait timed out");
    }

    // A time-out takes precedence over whatever the invalid products made happen next
    // (a failed factorisation, a stop, a non-converged eigenvalue).
    int iterate(FILE *out) override {
        int r = 0;
        try {
            r = iterate_body(out);
        } catch (const sdpg_error &e) {
            if (e.code != SDPG_ERR_TIMEOUT) check_tensor_timeout();
            throw;
        }
        if (r == 0) check_tensor_timeout();
        return r;
    }

    // one pass of pinpal's main loop body, sdpa_main.cpp:294-384
    int iterate_body(FILE *out) {
        if (!initialized_) initialize();
        if (stopped_) return 0;
        if (!(phase_updateCheck() && iter_ < par_.maxIteration)) return stop();
        direction_predictor();
        if (!newton(0)) return stop();
        step_length(0);
        direction_corrector();
        const R beta_rule = betaV_;
        const std::array<float, kPolIn> feat = policy_features(beta_rule);
        bool proposed = false;
        if (policy_ && (pol_flags_ & 1)) {
            float y[kPolOut];
            policy_eval(feat, y);
            betaV_ = R(std::min(1.0, std::max(0.01, (double)y[1])));
            proposed = true;
        }
        if (phase_ == pdFEAS && (beta_rule > R(5) || objP_ < objD_)) return stop();
        newton(1);
        step_length(1);
        if (proposed) {
            ++pol_props_;
            if (!proposal_ok()) {  // the fallback: the reference's own beta for this iteration
                ++pol_fallbacks_;
                const R delta = beta_rule - betaV_;
                betaV_ = beta_rule;
                newton_rebeta(delta);
                step_length(1);
            }
        }
        // the bounded waits of the tensor-core GEMMs and the Cholesky panels (step_length
        // has synchronised the streams)
        check_tensor_timeout();
        record_iteration();
        feats_.push_back(feat);
        lastAP_ = aP_;
        lastAD_ = aD_;
        print_iteration(out);
        trace_line();
        if (!update()) {
            cannot_move_ = true;
            return stop();
        }
        loop_after_update();
        return 1;
    }

    int stop() {
        stopped_ = true;
        return 0;
    }

    // ---------------------------------------------------------------- main-loop steps
    // (the C++ drop-in classes drive the loop through these, in pinpal's order)
    bool loop_phase_check() override {
        if (!initialized_) initialize();
        return phase_updateCheck();
    }
    void loop_direction(int corrector) override {
        if (corrector) direction_corrector();
        else direction_predictor();
    }
    bool loop_corrector_break() const override { return phase_ == pdFEAS && (betaV_ > R(5) || objP_ < objD_); }
    void loop_record(FILE *out, FILE *display) override {
        check_tensor_timeout();
        record_iteration();
        feats_.push_back(policy_features(betaV_));
        lastAP_ = aP_;
        lastAD_ = aD_;
        print_iteration(out);
        if (display) print_iteration_row(display, hist_.size() - 1);
    }
    bool loop_update() override {
        if (!update()) {
            cannot_move_ = true;
            return false;
        }
        return true;
    }
    void loop_after_update() override {
        // RatioInitResCurrentRes::update (sdpa_parts.cpp:692-698)
        if (reductionOn_) {
            thP_ = rabs((R(1.0) - aP_) * thP_);
            thD_ = rabs((R(1.0) - aD_) * thD_);
        }
        // AverageComplementarity::update (:647-651), Residuals::update
        muCur_ = ip_blocks(&Blk::X, &Blk::Z) / R(nDim_);
        residuals();
        // RatioInitResCurrentRes::update_exact (:700-708), SolveInfo::update
        thP_ = (initNormP_ > R(1.0e-10)) ? normP_ / initNormP_ : R(0.0);
        thD_ = (initNormD_ > R(1.0e-10)) ? normD_ / initNormD_ : R(0.0);
        solveInfo_update();
        ++iter_;
    }
    void loop_values(int *phase, int *iteration, void *out9) const override {
        *phase = phase_;
        *iteration = iter_;
        V *o = (V *)out9;
        const R vals[9] = {betaV_, objP_, objD_, muCur_, muInit_, aP_, aD_, thP_, thD_};
        for (int i = 0; i < 9; ++i) o[i] = vals[i].v;
    }
    void loop_finish(FILE *out, FILE *display) override {
        if (cannot_move_ && display) fprintf(display, "cannot move\n");
        residuals();
        final_phase_ = reverse_phase(phase_);
        print_last(out);
        print_last(display);
    }

    // pinpal's main loop, sdpa_main.cpp:294-385
    int run(FILE *out, FILE *display) override {
        auto t0 = std::chrono::steady_clock::now();
        if (!initialized_) initialize();
        const char *hdr = "   mu      thetaP  thetaD  objP      objD      alphaP  alphaD  beta \n";
        if (out) fputs(hdr, out);
        if (display) fputs(hdr, display);
        while (true) {
            const size_t before = hist_.size();
            const int r = iterate(out);
            if (display && hist_.size() > before) print_iteration_row(display, hist_.size() - 1);
            if (!r) break;
        }
        if (cannot_move_ && display) fprintf(display, "cannot move\n");
        residuals();
        final_phase_ = reverse_phase(phase_);
        tm_.total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        print_last(out);
        print_last(display);
        return iter_;
    }

    void print_iteration_row(FILE *f, size_t i) {
        if (!f || i >= printed_.size()) return;
        fputs(printed_[i].c_str(), f);
        fflush(f);
    }

    static int reverse_phase(int ph) {
        switch (ph) {
            case pFEAS: return dFEAS;
            case dFEAS: return pFEAS;
            case pFEAS_dINF: return pINF_dFEAS;
            case pINF_dFEAS: return pFEAS_dINF;
            case pUNBD: return dUNBD;
            case dUNBD: return pUNBD;
        }
        return ph;
    }

    // values of IO::printLastInfo (sdpa_io.cpp:996-1184), REVERSE_PRIMAL_DUAL branch
    R relgap() const {
        const R mean = (rabs(objP_) + rabs(objD_)) / R(2.0);
        const R PDgap = rabs(objP_ - objD_);
        return (mean < R(1.0)) ? PDgap : PDgap / mean;
    }
    R digits() const {
        const R mean = (rabs(objP_) + rabs(objD_)) / R(2.0);
        const R PDgap = rabs(objP_ - objD_);
        if (PDgap == R(0.0) || mean == R(0.0)) return R(0.0);
        return R(-log10(fabs((PDgap / mean).d())));
    }

    void print_last(FILE *f) {
        if (!f) return;
        print_iteration(f);
        fprintf(f, "\nphase.value = %s\n", phase_name(final_phase_));
        fprintf(f, "   Iteration = %d\n", iter_);
        fprintf(f, "          mu = %s\n", muCur_.fmt(16).c_str());
        fprintf(f, "relative gap = %s\n", relgap().fmt(16).c_str());
        fprintf(f, "         gap = %s\n", (muCur_ * R(nDim_)).fmt(16).c_str());
        fprintf(f, "      digits = %s\n", digits().fmt(16).c_str());
        fprintf(f, "objValPrimal = %s\n", (-objD_).fmt(16).c_str());
        fprintf(f, "objValDual   = %s\n", (-objP_).fmt(16).c_str());
        fprintf(f, "p.feas.error = %s\n", normD_.fmt(16).c_str());
        fprintf(f, "d.feas.error = %s\n", normP_.fmt(16).c_str());
        fprintf(f, "relative eps = %s\n", R(ml_ldexp(ml_one<N>(), -32 * N)).fmt(16).c_str());
        fprintf(f, "total time   = %.3f\n", tm_.total / 1000.0);
        fflush(f);
    }

    // The rest of IO::printLastInfo's file output (sdpa_io.cpp:1152-1173): the parameter
    // block (Parameter::display, sdpa_parts.cpp:227-255), the time table
    // (ComputeTime::display, sdpa_parts.cpp:72-122) and the solution with the
    // REVERSE_PRIMAL_DUAL naming: xVec = -y, xMat = Z, yMat = X, each through its format.
    void print_result_tail(FILE *f, double file_read_s) override {
        if (!f) return;
        fprintf(f, "\n\nParameters are\n");
        fprintf(f, "** Parameters **\n");
        fprintf(f, "maxIteration =    %d\n", par_.maxIteration);
        fprintf(f, "epsilonStar  = %8.3e\n", par_.epsilonStar);
        fprintf(f, "lambdaStar   = %8.3e\n", par_.lambdaStar);
        fprintf(f, "omegaStar    = %8.3e\n", par_.omegaStar);
        fprintf(f, "lowerBound   = %8.3e\n", par_.lowerBound);
        fprintf(f, "upperBound   = %8.3e\n", par_.upperBound);
        fprintf(f, "betaStar     = %8.3e\n", par_.betaStar);
        fprintf(f, "betaBar      = %8.3e\n", par_.betaBar);
        fprintf(f, "gammaStar    = %8.3e\n", par_.gammaStar);
        fprintf(f, "epsilonDash  = %8.3e\n", par_.epsilonDash);
        fprintf(f, "precision    =    %d\n", par_.precision);
        fprintf(f, "xPrint       = %s \n", par_.xPrint.c_str());
        fprintf(f, "XPrint       = %s \n", par_.XPrint.c_str());
        fprintf(f, "YPrint       = %s \n", par_.YPrint.c_str());
        fprintf(f, "infPrint     = %s \n", par_.infPrint.c_str());
        // time table: this solver's phase timers under the reference's row names; rows it
        // does not time separately print zero
        const double loop = tm_.total / 1000.0;
        const double bmat = tm_.schur / 1000.0;
        const std::pair<const char *, double> rows[] = {
            {" Predictor time  ", 0.0},           {" Corrector time  ", 0.0},
            {" Make bMat time  ", bmat},          {" Make bDia time  ", 0.0},
            {" Make bF1  time  ", 0.0},           {" Make bF2  time  ", 0.0},
            {" Make bF3  time  ", 0.0},           {" Make bPRE time  ", 0.0},
            {" Make rMat time  ", 0.0},           {" Make gVec Mul   ", 0.0},
            {" Make gVec time  ", tm_.rmat_gvec / 1000.0},
            {" Cholesky bMat   ", tm_.cholesky / 1000.0},
            {" Ste Pre time    ", 0.0},           {" Ste Cor time    ", tm_.steplen / 1000.0},
            {" solve           ", 0.0},           {" sumDz           ", 0.0},
            {" makedX          ", 0.0},           {" symmetriseDx    ", 0.0},
            {" makedXdZ        ", tm_.dxdz / 1000.0},
            {" xMatTime        ", 0.0},           {" zMatTime        ", 0.0},
            {" invzMatTime     ", 0.0},           {" xMatzMatTime    ", tm_.update / 1000.0},
            {" EigxMatTime     ", 0.0},           {" EigzMatTime     ", 0.0},
            {" EigxMatzMatTime ", 0.0},           {" updateRes       ", tm_.residual / 1000.0},
            {" EigTime         ", 0.0},           {" sub_total_bMat  ", loop - bmat},
            {" Main Loop       ", loop},          {" File Check      ", 0.0},
            {" File Change     ", 0.0},           {" File Read       ", file_read_s},
            {" Total           ", loop + file_read_s}};
        fprintf(f, "\n");
        fprintf(f, "                         Time(sec) ");
        fprintf(f, " Ratio(%% : MainLoop) \n");
        for (const auto &r : rows) fprintf(f, "%s=       %f,  %f\n", r.first, r.second, r.second / loop * 100.0);
        fprintf(f, "\n");
        // solution
        fprintf(f, "xVec = \n");
        {
            std::vector<V> h(m_);
            d2h_ += (long long)m_ * (long long)sizeof(V);
            SDPG_CUDA(cudaMemcpyAsync(h.data(), y_, m_ * sizeof(V), cudaMemcpyDeviceToHost, st_));
            SDPG_CUDA(cudaStreamSynchronize(st_));
            if (par_.xPrint == "NOPRINT") {
                fprintf(f, "NOPRINT\n");
            } else {
                fprintf(f, "{");
                for (int i = 0; i < m_; ++i) {
                    fputs(ml_format_gmp<N>(par_.xPrint, ml_neg(h[i])).c_str(), f);
                    fputs(i + 1 < m_ ? "," : "}\n", f);
                }
                if (m_ == 0) fprintf(f, "  }\n");
            }
        }
        fprintf(f, "xMat = \n");
        print_blocks(f, &Blk::Z, par_.XPrint);
        fprintf(f, "yMat = \n");
        print_blocks(f, &Blk::X, par_.YPrint);
    }
    // IO::displayDenseLinarSpaceLast (sdpa_io.cpp:1186-1220) with DenseMatrix::display
    // (sdpa_struct.cpp:706-746) for every block, column-major entries
    void print_blocks(FILE *f, V *Blk::*M, const std::string &fmt) const {
        if (fmt == "NOPRINT") {
            fprintf(f, "NOPRINT\n");
            return;
        }
        fprintf(f, "{\n");
        for (const Blk &B : blk_) {
            const int n = B.n;
            std::vector<V> h((size_t)n * n);
            d2h_ += (long long)h.size() * (long long)sizeof(V);
            SDPG_CUDA(cudaMemcpyAsync(h.data(), B.*M, h.size() * sizeof(V), cudaMemcpyDeviceToHost, st_));
            SDPG_CUDA(cudaStreamSynchronize(st_));
            auto at = [&](int i, int j) { return ml_format_gmp<N>(fmt, h[i + (size_t)n * j]); };
            if (B.lp) {  // an LP block prints its diagonal as one braced row
                fprintf(f, "{");
                for (int k = 0; k < n; ++k) {
                    fputs(at(k, k).c_str(), f);
                    fputs(k + 1 < n ? "," : "}\n", f);
                }
                continue;
            }
            fprintf(f, "{");
            for (int i = 0; i + 1 < n; ++i) {
                fputs(i == 0 ? " {" : "  {", f);
                for (int j = 0; j < n; ++j) {
                    fputs(at(i, j).c_str(), f);
                    fputs(j + 1 < n ? "," : " },\n", f);
                }
            }
            if (n > 1) fputs("  {", f);
            for (int j = 0; j < n; ++j) {
                fputs(at(n - 1, j).c_str(), f);
                fputs(j + 1 < n ? "," : " }", f);
            }
            fputs(n > 1 ? "   }\n" : "\n", f);
        }
        fprintf(f, "}\n");
    }

    // info: [phase, iteration, objValPrimal, objValDual, mu, relgap, p.feas.error, d.feas.error,
    //        alphaP, alphaD, beta, digits] as printed by the reference (primal/dual swapped back)
    void info(double *o) const override {
        o[0] = final_phase_;
        o[1] = iter_;
        o[2] = (-objD_).d();
        o[3] = (-objP_).d();
        o[4] = muCur_.d();
        o[5] = relgap().d();
        o[6] = normD_.d();
        o[7] = normP_.d();
        o[8] = aD_.d();
        o[9] = aP_.d();
        o[10] = betaV_.d();
        o[11] = digits().d();
    }
    std::string info_text(int which, int digits_) const override {
        switch (which) {
            case 0: return (-objD_).fmt(digits_ - 1);
            case 1: return (-objP_).fmt(digits_ - 1);
            case 2: return muCur_.fmt(digits_ - 1);
            case 3: return relgap().fmt(digits_ - 1);
            case 4: return normD_.fmt(digits_ - 1);
            case 5: return normP_.fmt(digits_ - 1);
        }
        return "";
    }
    // The reference prints xVec = -y (IO::printLastInfo, Vector::display with scalar -1).
    void get_y(void *out, int form) const override {
        std::vector<V> h(m_);
        d2h_ += (long long)m_ * (long long)sizeof(V);
        SDPG_CUDA(cudaMemcpyAsync(h.data(), y_, m_ * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < m_; ++i) {
            if (form == 0) ((double *)out)[i] = ml_to_double(ml_neg(h[i]));
            else ((V *)out)[i] = ml_neg(h[i]);
        }
    }
    void get_block(int which, int l, void *out, int form) const override {
        const Blk &B = blk_.at(l);
        const size_t nn = (size_t)B.n * B.n;
        std::vector<V> h(nn);
        const V *srcs[] = {B.X, B.Z, B.Dx, B.Dz, B.Zinv, B.LX, B.LZ, B.C, B.Dres};
        if (which < 0 || which > 8) throw sdpg_error(SDPG_ERR_ARG, "bad matrix selector");
        const V *src = srcs[which];
        d2h_ += (long long)(nn * sizeof(V));
        SDPG_CUDA(cudaMemcpyAsync(h.data(), src, nn * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
        for (size_t i = 0; i < nn; ++i) {
            if (form == 0) ((double *)out)[i] = ml_to_double(h[i]);
            else ((V *)out)[i] = h[i];
        }
    }

    void make_bmat(void *out) override {
        Make_bMat();
        SDPG_CUDA(cudaMemcpyAsync(out, B_, (size_t)m_ * m_ * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
    }
    void make_gvec(int corrector, void *out) override {
        Make_gVec(corrector != 0);
        SDPG_CUDA(cudaMemcpyAsync(out, g_, m_ * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
    }
    void min_eigen(int side, void *out) override {
        const R v = side == 0 ? getMinEigen(&Blk::LX, &Blk::Dx) : getMinEigen(&Blk::LZ, &Blk::Dz);
        memcpy(out, &v.v, sizeof(V));
    }
    void get_vec(int which, void *out) const override {
        const V *srcs[] = {y_, Dy_, b_, p_};
        if (which < 0 || which > 3) throw sdpg_error(SDPG_ERR_ARG, "bad vector selector");
        SDPG_CUDA(cudaMemcpyAsync(out, srcs[which], m_ * sizeof(V), cudaMemcpyDeviceToHost, st_));
        SDPG_CUDA(cudaStreamSynchronize(st_));
    }

    // ---------------------------------------------------------------- timing

    void ev_start() { SDPG_CUDA(cudaEventRecord(ev_[0], st_)); }
    double ev_stop() {
        SDPG_CUDA(cudaEventRecord(ev_[1], st_));
        SDPG_CUDA(cudaEventSynchronize(ev_[1]));
        float ms = 0;
        SDPG_CUDA(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
        return ms;
    }

  private:
    Param par_;
    double lambda_default_;  // param.sdpa's lambdaStar (a proposal replaces par_'s copy)
    int dev_;
    cudaStream_t st_;
    Workspace ws_, ws2_;  // ws2_ serves work issued on the second stream
    int *tc_error_ = nullptr;  // device word: a tensor-core GEMM or Cholesky panel gave up a bounded wait

    cudaStream_t st2_ = nullptr;
    cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
    static constexpr int kPinned = 4096;
    V *pinned_ = nullptr;  // page-locked staging for per-step scalars
    int *info2_ = nullptr, *info_all_ = nullptr;
    std::vector<Blk> blk_;
    int m_ = 0, nDim_ = 0;
    std::vector<V> b_h_;
    V *BLinv_ = nullptr, *BLinvT_ = nullptr, *Dytmp_ = nullptr;  // inverse of the Schur factor and its transpose
    V *b_ = nullptr, *y_ = nullptr, *Dy_ = nullptr, *g_ = nullptr, *p_ = nullptr, *B_ = nullptr, *slot_ = nullptr;
    int *info_ = nullptr, *status_ = nullptr;
    R muInit_, muCur_, thP_, thD_, aP_, aD_, betaV_, rho_, etaP_, etaD_, objP_, objD_, normP_, normD_;
    R initNormP_, initNormD_;
    int phase_ = noINFO, final_phase_ = noINFO, reductionOn_ = 1, iter_ = 0;
    bool initialized_ = false, stopped_ = false, cannot_move_ = false;
    std::vector<std::string> printed_;
    Timers tm_;
    std::vector<IterRecord> hist_;
    std::vector<cudaEvent_t> ev_;
    FILE *trace_ = nullptr;
    long long gemm_macs_ = 0;
    bool prof_on_ = false;
    std::vector<cudaEvent_t> prof_ev_;
    int prof_used_ = 0;
    double prof_ms_ = 0;
    long long prof_launches_ = 0, prof_macs_ = 0;
    mutable long long h2d_ = 0, d2h_ = 0;
    bool has_init_ = false;  // an initial point replaces lambdaStar * I
    InitPoint init_;
    // learned proposal
    const Policy *policy_ = nullptr;
    int pol_flags_ = 0;
    float *pol_dev_ = nullptr;  // device: inputs at 0, outputs at 8
    long long pol_props_ = 0, pol_fallbacks_ = 0;
    double pol_lambda_prop_ = 0;
    R lastAP_, lastAD_;
    std::vector<std::array<float, kPolIn>> feats_;
};

}  // namespace

SolverBase *make_solver(const RawProblem &P, const Param &param, int device, cudaStream_t stream) {
    const int bits = param.precision;
    if (bits <= 256) return new Solver<8>(P, param, device, stream);
    if (bits <= 512) return new Solver<16>(P, param, device, stream);
    throw sdpg_error(SDPG_ERR_ARG, "precision above 512 bits is not supported");
}

}  // namespace sdpg
