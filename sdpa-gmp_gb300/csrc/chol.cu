// Cholesky factorisation, triangular inverse and triangular solves in
// multi-limb arithmetic (replacing Rpotrf / Rtrsm / Rtrsv as called from
// Lal::choleskyFactorWithAdjust, Lal::getCholesky, Lal::getInvLowTriangularMatrix
// and Lal::solveSystems, sdpa_linear.cpp:342-455, 608-695).
//
// Blocked left-looking with 32-wide panels: each panel first receives the product of
// the finished columns (the residue-path GEMM), then one cluster launch factors its
// diagonal block and, a step behind, the rows below it, all by the same division-free
// elimination with full multi-limb pivots.
#include <cooperative_groups.h>

#include "kernels.cuh"
#include "mlfix.cuh"
#include "mlwarp.cuh"
#include "tc_gemm.cuh"
#include "tcgen05.cuh"

namespace cg = cooperative_groups;

namespace sdpg {

namespace {

constexpr int NB = 32;

// One launch factors a whole 32-column panel: the kb x kb diagonal block and the rows
// below it.
//
// Division-free elimination.  Every entry of the panel's lower part is held in a
// register by its own thread.  Step j updates every entry right of column j as
//     s_it <- (p_j s_it - s_ij s_tj) * 2^-e_j,     p_j = s_jj in [2^(e_j-1), 2^e_j),
// so S^(j) = c_j T^(j) where T^(j) is the usual Schur complement and
// c_{j+1} = c_j p_j 2^-e_j.  No square root or reciprocal sits on the pivot chain; at
// the end every column is normalised at once with L[i][t] = s_it / sqrt(c_t p_t).
//
// The diagonal block (528 entries, numbered column by column: column t holds rows
// t..NB-1) is spread over a cluster of C CTAs (one per SM), entry q in CTA q mod C.  The
// entries still active at step j (t > j) are the highest-numbered ones, so in every CTA
// whole warps drop out as the elimination proceeds while the remaining work stays spread
// over all C SMs.  Every CTA keeps a copy of the columns (column j as it stands at step
// j, when it holds the pivot): an entry that becomes final stores itself into all copies
// with st.async, and each column's mbarrier tells a CTA when the column has arrived.  A
// thread waits only for the columns it reads, so a step costs one update and one remote
// store instead of the slowest thread's update plus a cluster barrier.
//
// The rows below take the same steps one warp per row (lane t holds s_it): s_ij is lane
// j of the same warp and p_j, s_tj (column j of the diagonal block after j steps) come
// from a history buffer in global memory that one warp of the diagonal cluster fills as
// the columns arrive, behind a progress word.  So the rows run a few steps behind the
// diagonal block rather than after it, and no separate triangular solve follows.
//
// Roles: each cluster draws a ticket when it starts; the first factors the diagonal
// block, so a cluster that waits always waits on one that is running.  The row waits
// are bounded by a cycle budget: on time-out the row sets *info = -1 (if it was 0) and
// the error word, and returns (the diagonal block's own waits have the full budget and
// do the same).
//
// info: 0, or (col0 + j + 1) for the first non-positive pivot.
// sync (two ints, zeroed once per factorisation): [0] ticket counter, [1] progress, which
// for the panel with progress base `base` reads base + j + 1 once hist column j is out,
// base + kPanelFinal once the normalisers are, and base + kPanelAbort after a bad pivot.
// hist: NB x NB entries (column j at hist[j NB ..]), then the NB normalisers.
constexpr int kPanelFinal = 40;
constexpr int kPanelAbort = 63;
constexpr int kPanelTimeout = 6;                 // error-word code of a panel wait that gave up
constexpr long long kPanelWaitCycles = 1ll << 31;  // about one second at 2 GHz
static_assert(kPanelAbort < 64 && kPanelFinal > NB, "progress values of one panel stay below the next base");

// Launch shape for a cluster of C CTAs: the entries of the diagonal block dealt out
// cyclically (entry q to CTA q mod C, local index q / C), so at every step the active
// entries (the highest-numbered ones) are spread evenly over the cluster's SMs, and one
// more warp per CTA, which holds no entry (in CTA 0 it fills the history).  A CTA of a
// row cluster works R rows, one per warp, and its other warps leave.
template <int C>
struct PanelShape {
    static constexpr int per_cta = (NB * (NB + 1) / 2 + C - 1) / C;
    static constexpr int threads = ((per_cta + 31) / 32 + 1) * 32;
};
constexpr int kPanelCluster = 4;  // cluster size of ml_potrf's panels
constexpr int kPanelRowWarps = 4;  // rows per CTA of the row clusters (at most threads / 32)

template <int N>
__device__ __forceinline__ mlf<N> ml_load_cg(const mlf<N> *p) {
    mlf<N> r;
    const unsigned *w = reinterpret_cast<const unsigned *>(p);
    unsigned *o = reinterpret_cast<unsigned *>(&r);
#pragma unroll
    for (int k = 0; k < N + 2; ++k) o[k] = __ldcg(w + k);
    return r;
}

// one multi-limb value in shared memory, padded to the 16-byte unit of st.async
template <int N>
struct alignas(16) PanelSlot {
    mlf<N> v;
};

// packed column-major lower triangle with the diagonal: column t holds rows t..NB-1
__host__ __device__ constexpr int packed_col(int i, int t) { return NB * t - t * (t - 1) / 2 + (i - t); }

// the shared::cluster address of a shared-memory location of CTA `rank`
__device__ __forceinline__ uint32_t cluster_addr(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

// v into the cluster shared-memory address dst (16-byte aligned), completing its
// sizeof(mlf<N>) bytes on the mbarrier at bar (same CTA as dst)
template <int N>
__device__ __forceinline__ void st_async_ml(uint32_t dst, const mlf<N> &v, uint32_t bar) {
    constexpr int W = (int)sizeof(mlf<N>) / 4;  // 10 or 18 words: 16-byte pieces, then 8
    static_assert(W % 4 == 2, "layout of mlf");
    const uint32_t *w = reinterpret_cast<const uint32_t *>(&v);
#pragma unroll
    for (int k = 0; k + 4 <= W; k += 4)
        asm volatile(
            "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                dst + 4u * k),
            "r"(w[k]), "r"(w[k + 1]), "r"(w[k + 2]), "r"(w[k + 3]), "r"(bar)
            : "memory");
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];" ::"r"(
                     dst + 4u * (W - 2)),
                 "r"(w[W - 2]), "r"(w[W - 1]), "r"(bar)
                 : "memory");
}

// the calling warp's history stores, then the progress word (one warp, all lanes)
__device__ __forceinline__ void panel_progress(int *prog, int v) {
    __threadfence();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) atomicExch(prog, v);
}

// wait (all lanes of a warp) until *prog >= target; the value seen, or -1 on time-out
__device__ __forceinline__ int panel_wait(const int *prog, int target, long long budget) {
    int v = *(volatile const int *)prog;
    if (v < target) {
        const long long t0 = clock64();
        while ((v = *(volatile const int *)prog) < target) {
            if (clock64() - t0 > budget) return -1;
            __nanosleep(32);
        }
    }
    __threadfence();
    return v;
}

template <int N, int C, int R>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(PanelShape<C>::threads)
    panel_factor_kernel(mlf<N> *A, int lda, int col0, int kb, int rows, int *info, mlf<N> *hist, int *sync, int base,
                        int ticket0, long long budget, int *err) {
    __shared__ PanelSlot<N> colv[NB * (NB + 1) / 2];      // column j of S^(j) at colv[packed_col(i, j)]
    __shared__ __align__(8) unsigned long long bars[NB];  // bars[j]: column j has arrived here
    __shared__ mlf<N> cs[NB];                             // c_j
    __shared__ mlf<N> rs[NB];                             // 1/sqrt(c_j p_j)
    __shared__ int role[2];  // rank 0: this cluster's ticket in the launch, *info at start
    __shared__ int status;   // thread 0: 0, the failing column's info value, or -1 (a wait gave up)
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int lane = threadIdx.x & 31;
    int *prog = sync + 1;
    const uint32_t colv0 = tc::smem_u32(colv), bars0 = tc::smem_u32(bars);
    if (threadIdx.x == 0) {  // column j brings kb - j entries into every CTA of the cluster
        for (int j = 0; j < kb; ++j) tc::mbar_init(bars0 + 8u * j, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int j = 0; j < kb; ++j) tc::mbar_expect_tx(bars0 + 8u * j, (kb - j) * (uint32_t)sizeof(mlf<N>));
    }
    if (rank == 0 && threadIdx.x == 0) {
        role[0] = atomicAdd(&sync[0], 1) - ticket0;
        role[1] = *(volatile int *)info;
    }
    cluster.sync();  // also: every CTA's barriers are initialised before any remote store
    const int tk = *cluster.map_shared_rank(&role[0], 0);
    const int info0 = *cluster.map_shared_rank(&role[1], 0);
    cluster.sync();     // rank 0's words are read before any CTA of the cluster leaves
    if (info0 != 0) return;  // an earlier panel failed: the whole launch leaves

    if (tk > 0) {  // ------------------------------------------------ rows below the block
        const int w = (int)(threadIdx.x >> 5);
        const int r = (tk - 1) * C * R + rank * R + w;
        if (w >= R || r >= rows) return;
        mlf<N> *row = A + col0 + kb + r + (long long)col0 * lda;  // entry t at row[t * lda]
        mlf<N> a = lane < kb ? row[(long long)lane * lda] : ml_zero<N>();
        int seen = 0;
        // p_j and s_tj of the next step, loaded a step early whenever the progress word
        // already showed them (the rows trail the diagonal block, so mostly they are)
        mlf<N> pn = ml_zero<N>(), sn = ml_zero<N>();
        bool have = false;
        for (int j = 0; j <= kb; ++j) {
            const int need = j + 1 < kb ? base + j + 1 : base + kPanelFinal;
            if (!have && seen < need) {
                seen = panel_wait(prog, need, budget);
                if (seen < 0) {
                    if (lane == 0) {
                        atomicCAS(info, 0, -1);
                        atomicExch(err, kPanelTimeout);
                    }
                    return;
                }
                if (seen >= base + kPanelAbort) return;  // the diagonal block failed
            }
            if (j + 1 >= kb) break;  // normalisers published
            if (!have) {
                pn = ml_load_cg(hist + (long long)j * NB + j);
                sn = lane > j && lane < kb ? ml_load_cg(hist + (long long)j * NB + lane) : ml_zero<N>();
            }
            const mlf<N> p = pn, stj = sn;
            have = j + 2 < kb && seen >= base + j + 2 && seen < base + kPanelAbort;
            if (have) {
                pn = ml_load_cg(hist + (long long)(j + 1) * NB + j + 1);
                sn = lane > j + 1 && lane < kb ? ml_load_cg(hist + (long long)(j + 1) * NB + lane) : ml_zero<N>();
            }
            const mlf<N> sij = ml_shfl(a, j);
            if (lane > j && lane < kb) a = ml_ldexp(ml_sub(ml_mul(p, a), ml_mul(sij, stj)), -p.e);
        }
        if (lane < kb) row[(long long)lane * lda] = ml_mul(a, ml_load_cg(hist + NB * NB + lane));
        return;
    }

    // ---------------------------------------------------------------- the diagonal block
    mlf<N> *Akk = A + col0 + (long long)col0 * lda;
    const bool signal = rank == 0 && (int)threadIdx.x >= PanelShape<C>::threads - 32;  // fills hist
    const int q = (int)threadIdx.x * C + rank;  // packed_col(i, t) of this thread's entry
    int t = 0;
    while (t + 1 < NB && NB * (t + 1) - (t + 1) * t / 2 <= q) ++t;
    const int i = t + (q - (NB * t - t * (t - 1) / 2));  // entry (i, t), t <= i
    const bool mine = (int)threadIdx.x < PanelShape<C>::per_cta && q < NB * (NB + 1) / 2 && i < kb;
    mlf<N> a = mine ? Akk[i + (long long)t * lda] : ml_zero<N>();
    // v into slot q of every CTA, completing bars[col] there
    auto publish = [&](const mlf<N> &v, int col) {
#pragma unroll
        for (int r = 0; r < C; ++r)
            st_async_ml<N>(cluster_addr(colv0 + q * (uint32_t)sizeof(PanelSlot<N>), r), v,
                           cluster_addr(bars0 + 8u * col, r));
    };
    if (mine && t == 0) publish(a, 0);
    // thread 0 of every CTA follows every column: it carries c_j and the status
    const int steps = threadIdx.x == 0 ? kb : (mine ? t : 0);
    mlf<N> c = ml_one<N>();
    int bad = 0;
    for (int j = 0; j < steps; ++j) {
        if (!tc::mbar_wait_acq_cluster(bars0 + 8u * j, 0, kPanelWaitCycles)) {
            bad = -1;
            break;
        }
        const mlf<N> p = colv[packed_col(j, j)].v;
        if (ml_sign(p) <= 0) {
            bad = col0 + j + 1;
            break;
        }
        if (threadIdx.x == 0) {
            cs[j] = c;
            c = ml_mul(c, ml_ldexp(p, -p.e));
        }
        if (mine && t > j) {  // (thread 0 runs every step for c_j; its own entry is in column 0)
            const mlf<N> u = ml_sub(ml_mul(p, a), ml_mul(colv[packed_col(i, j)].v, colv[packed_col(t, j)].v));
            a = ml_ldexp(u, -p.e);
            if (t == j + 1) publish(a, t);
        }
    }
    if (signal) {  // hist column j as soon as it is here, behind the progress word
        for (int j = 0; j + 1 < kb; ++j) {
            if (!tc::mbar_wait_acq_cluster(bars0 + 8u * j, 0, kPanelWaitCycles)) break;
            if (ml_sign(colv[packed_col(j, j)].v) <= 0) break;
            if (lane >= j && lane < kb) hist[(long long)j * NB + lane] = colv[packed_col(lane, j)].v;
            panel_progress(prog, base + j + 1);
        }
    }
    if (threadIdx.x == 0) status = bad;
    __syncthreads();
    bad = status;
    if (!bad) {
        if ((int)threadIdx.x < kb) {  // p_t is the diagonal entry of column t
            const mlf<N> pt = colv[packed_col(threadIdx.x, threadIdx.x)].v;
            rs[threadIdx.x] = ml_rsqrt(ml_mul(cs[threadIdx.x], pt));
        }
        __syncthreads();
        if (mine) Akk[i + (long long)t * lda] = ml_mul(a, rs[t]);
        if (signal) {
            if (lane < kb) hist[NB * NB + lane] = rs[lane];
            panel_progress(prog, base + kPanelFinal);
        }
    } else {
        if (rank == 0 && threadIdx.x == 0) {
            if (bad > 0) {
                *info = bad;
            } else {
                atomicCAS(info, 0, -1);
                atomicExch(err, kPanelTimeout);
            }
        }
        if (signal) panel_progress(prog, base + kPanelAbort);
    }
    cluster.sync();  // no CTA leaves while another may still write its shared memory
}

// The previous panel's share of panel k0's update, on the CUDA cores (the look-ahead
// product on the tensor cores has taken every earlier column):
//     A[i][k0 + t] -= sum_{m < 32} L[i][kc + m] L[k0 + t][kc + m],  i in [k0, n), t < kb,
// lower part of the diagonal block only.
//
// In block floating point (mlfix.cuh: each row's 32 values as 28-bit digits relative to
// the row's largest exponent, digit products summed exactly, one rounding per entry): the
// truncation is relative to 2^(E_i + E_t), about 2^-270 of sqrt(A_ii A_tt) for a Cholesky
// factor, the form of the factorisation's backward error.  The rows' digits go to shared
// memory as [m][digit][row] (a warp's 32 lanes read 32 consecutive words), the columns'
// as [t][m][digit] (one address per warp).
constexpr int kUpdCols = 4;  // columns t per CTA of the update kernel (two warps each)
constexpr int kUpdWarps = 2 * kUpdCols;

// dynamic shared memory of the update kernel: digits of 32 rows and kUpdCols columns,
// then the second warps' half-sums
template <int N>
constexpr size_t panel_update_smem() {
    return (size_t)(32 + kUpdCols) * 32 * BfpShape<N>::D * sizeof(int32_t) +
           (size_t)BfpShape<N>::NC * kUpdCols * 32 * sizeof(long long);
}

// CTA: 32 rows i (lane) x kUpdCols columns t, two warps per column, each summing 16 of
// the 32 terms; the second adds its exact column sums to the first's through shared
// memory.  Few columns per CTA spread the integer multiply-adds over many SMs.

template <int N>
__global__ void __launch_bounds__(32 * kUpdWarps) panel_update_kernel(mlf<N> *A, int lda, int n, int k0, int kb,
                                                                     int kc) {
    using B = BfpShape<N>;
    constexpr int D = B::D, NC = B::NC;
    constexpr int MW = NB / kUpdWarps;  // row values each warp converts
    extern __shared__ int32_t bfp_sm[];
    int32_t *di = bfp_sm;                // rows:    di[(m * D + p) * 32 + r]
    int32_t *dt = bfp_sm + 32 * 32 * D;  // columns: dt[(c * 32 + m) * D + p]
    long long *part = reinterpret_cast<long long *>(bfp_sm + (32 + kUpdCols) * 32 * D);  // [col][c][r]
    __shared__ int emax[kUpdWarps][32];  // partial row maxima
    __shared__ int et[kUpdCols];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i0 = k0 + (int)blockIdx.x * 32, t0 = (int)blockIdx.y * kUpdCols;
    constexpr int kNone = kBfpNone;
    // rows: lane = row, warp w takes m = MW w .. MW w + MW - 1
    const int ri = i0 + lane;
    mlf<N> xv[MW];
#pragma unroll
    for (int k = 0; k < MW; ++k) {
        const int m = MW * warp + k;
        xv[k] = ri < n ? A[ri + (long long)(kc + m) * lda] : ml_zero<N>();
    }
    int e = kNone;
#pragma unroll
    for (int k = 0; k < MW; ++k) e = xv[k].m[N - 1] ? max(e, xv[k].e) : e;
    emax[warp][lane] = e;
    // columns: warp w < kUpdCols reads column t0 + w, lane = m
    mlf<N> yv = ml_zero<N>();
    if (warp < kUpdCols) {
        const int tw = t0 + warp;
        yv = tw < kb ? A[k0 + tw + (long long)(kc + lane) * lda] : ml_zero<N>();
        int ey = yv.m[N - 1] ? yv.e : kNone;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ey = max(ey, __shfl_xor_sync(0xffffffffu, ey, o));
        if (lane == 0) et[warp] = ey;
    }
    __syncthreads();
    int Er = emax[0][lane];
#pragma unroll
    for (int w = 1; w < kUpdWarps; ++w) Er = max(Er, emax[w][lane]);
    const int tl = warp % kUpdCols, half = warp / kUpdCols;
    const int Ey = et[tl];
    {
        int32_t d[D];
#pragma unroll
        for (int k = 0; k < MW; ++k) {
            bfp_digits<N>(xv[k], Er, d);
            const int m = MW * warp + k;
#pragma unroll
            for (int p = 0; p < D; ++p) di[(m * D + p) * 32 + lane] = d[p];
        }
        if (warp < kUpdCols) {
            bfp_digits<N>(yv, Ey, d);
#pragma unroll
            for (int p = 0; p < D; ++p) dt[(warp * 32 + lane) * D + p] = d[p];
        }
    }
    __syncthreads();
    // entry (i0 + lane, t0 + tl); this warp's half of the terms
    const int i = i0 + lane, t = t0 + tl;
    const bool live = i < n && t < kb && i - k0 >= t;
    long long acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = 0;
    if (live) {
        for (int m = half * (NB / 2); m < (half + 1) * (NB / 2); ++m) {
            int32_t a[D], b[D];
#pragma unroll
            for (int p = 0; p < D; ++p) {
                a[p] = di[(m * D + p) * 32 + lane];
                b[p] = dt[(tl * 32 + m) * D + p];
            }
            bfp_term<N>(acc, a, b);
            if (m % B::EVERY == B::EVERY - 1) bfp_carry<NC>(acc);
        }
        if (half) {
#pragma unroll
            for (int c = 0; c < NC; ++c) part[(tl * NC + c) * 32 + lane] = acc[c];
        }
    }
    __syncthreads();
    if (!live || half) return;
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] += part[(tl * NC + c) * 32 + lane];  // both halves carried: no overflow
    const mlf<N> dot = bfp_result<N>(acc, Er, Ey);
    mlf<N> *cp = A + i + (long long)(k0 + t) * lda;
    *cp = ml_sub(*cp, dot);
}


// Invert every NB x NB diagonal block of the lower-triangular L (n a multiple of NB)
// into Linv, one cluster of kPanelCluster CTAs per block and one thread per
// lower-triangle entry of the inverse, dealt cyclically over the cluster as in
// panel_factor_kernel.  Row-oriented substitution X = T^-1: entry (i, c) subtracts
// T[i][j] X[j][c] for j = c .. i-1 as each row j of X arrives, scales by 1/T[i][i], and
// stores X[i][c] into every CTA of the cluster with st.async, completing row i's
// mbarrier there: a thread waits only for the rows it reads, no barrier per step.
// T is read through the cache, each next value loaded before the wait for its row.
// A wait that gives up (about a second) sets *err to kTrtriTimeout; the rows it should
// have produced are then not written.
constexpr int kTrtriTimeout = 7;

// packed row-major lower triangle with the diagonal: row i holds columns 0..i
__host__ __device__ constexpr int packed_row(int i, int c) { return i * (i + 1) / 2 + c; }

template <int N>
__global__ void __cluster_dims__(kPanelCluster, 1, 1) __launch_bounds__(PanelShape<kPanelCluster>::threads)
    trtri_diag_kernel(const mlf<N> *L, int ldl, mlf<N> *Linv, int ldi, int *err) {
    constexpr int C = kPanelCluster;
    __shared__ mlf<N> rv[NB];                             // 1 / T[i][i]
    __shared__ PanelSlot<N> xr[NB * (NB + 1) / 2];        // X[i][c] at packed_row(i, c)
    __shared__ __align__(8) unsigned long long bars[NB];  // bars[i]: row i of X has arrived
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int o = (int)(blockIdx.x / C) * NB;
    const mlf<N> *T = L + o + (long long)o * ldl;
    mlf<N> *X = Linv + o + (long long)o * ldi;
    const uint32_t xr0 = tc::smem_u32(xr), bars0 = tc::smem_u32(bars);
    if (threadIdx.x == 0) {  // row i brings i + 1 entries into every CTA
        for (int r = 0; r < NB; ++r) tc::mbar_init(bars0 + 8u * r, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int r = 0; r < NB; ++r) tc::mbar_expect_tx(bars0 + 8u * r, (r + 1) * (uint32_t)sizeof(mlf<N>));
    }
    if (threadIdx.x < NB) rv[threadIdx.x] = ml_recip(T[threadIdx.x + (long long)threadIdx.x * ldl]);
    __syncthreads();
    cluster.sync();  // every CTA's barriers are initialised before any remote store
    const int q = (int)threadIdx.x * C + rank;  // packed_row(i, c) of this thread's entry
    int i = 0;
    while (i + 1 < NB && packed_row(i + 1, 0) <= q) ++i;
    const int c = q - packed_row(i, 0);
    const bool mine = (int)threadIdx.x < PanelShape<C>::per_cta && q < NB * (NB + 1) / 2;
    mlf<N> x = ml_zero<N>();
    bool ok = true;
    if (mine) {
        x = i == c ? ml_one<N>() : ml_zero<N>();
        mlf<N> tn = c < i ? T[i + (long long)c * ldl] : ml_zero<N>();
        for (int j = c; j < i; ++j) {
            const mlf<N> tj = tn;
            if (j + 1 < i) tn = T[i + (long long)(j + 1) * ldl];
            if (!tc::mbar_wait_acq_cluster(bars0 + 8u * j, 0, kPanelWaitCycles)) {
                ok = false;
                break;
            }
            x = ml_sub(x, ml_mul(tj, xr[packed_row(j, c)].v));
        }
        if (ok) {
            x = ml_mul(x, rv[i]);
#pragma unroll
            for (int r = 0; r < C; ++r)
                st_async_ml<N>(cluster_addr(xr0 + q * (uint32_t)sizeof(PanelSlot<N>), r), x,
                               cluster_addr(bars0 + 8u * i, r));
        } else {
            atomicExch(err, kTrtriTimeout);
        }
    }
    // every row stored into this CTA has arrived before it leaves (bounded)
    if (threadIdx.x == 0)
        for (int r = 0; r < NB; ++r)
            if (!tc::mbar_wait_acq_cluster(bars0 + 8u * r, 0, kPanelWaitCycles)) {
                atomicExch(err, kTrtriTimeout);
                break;
            }
    __syncthreads();
    cluster.sync();
    if (mine && ok) X[i + (long long)c * ldi] = x;
}

// Inverses of the NB x NB diagonal blocks of the lower-triangular L, packed:
// Dinv[b] (ld NB, lower, zeros above) = L[bNB:, bNB:]^{-1} restricted to the block.
template <int N>
__global__ void trtri_diag_packed_kernel(const mlf<N> *L, int ldl, mlf<N> *Dinv, int n) {
    const int b = blockIdx.x;
    const int o = b * NB;
    const int kb = min(NB, n - o);
    const mlf<N> *T = L + o + (long long)o * ldl;
    mlf<N> *X = Dinv + (long long)b * NB * NB;
    __shared__ mlf<N> rv[NB];
    if (threadIdx.x < kb) rv[threadIdx.x] = ml_recip(T[threadIdx.x + (long long)threadIdx.x * ldl]);
    for (int q = threadIdx.x; q < NB * NB; q += blockDim.x) {
        const int i = q % NB, c = q / NB;
        X[i + NB * c] = (i == c && i < kb) ? ml_one<N>() : ml_zero<N>();
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        for (int c = threadIdx.x; c <= j; c += blockDim.x) X[j + NB * c] = ml_mul(X[j + NB * c], rv[j]);
        __syncthreads();
        const int rows = kb - j - 1, cols = j + 1;
        for (int q = threadIdx.x; q < rows * cols; q += blockDim.x) {
            const int i = j + 1 + q % rows, c = q / rows;
            mlf<N> *x = X + i + NB * c;
            *x = ml_sub(*x, ml_mul(T[i + (long long)j * ldl], X[j + NB * c]));
        }
        __syncthreads();
    }
}

// Triangular solves as a wavefront over 32-row blocks, one CTA per block.  A CTA
// draws a ticket at start (so every CTA it waits on has already started and is
// resident), takes the contribution of each earlier block as soon as that block's
// solution is published, and publishes its own after the diagonal solve with the
// inverted diagonal block.  Only the last contribution and the diagonal solve are
// on the critical path.  Every wait is bounded: on time-out the CTA records
// status 1 and leaves (the result is then invalid and the caller reports it).
//
// sync (ints, zeroed before each launch): [0] ticket counter, [1 + b] block b done.
constexpr int kTrsvThreads = 256;

constexpr int kTrsvWarps = kTrsvThreads / 32;
constexpr long long kSpinLimit = 1ll << 24;

__device__ __forceinline__ bool wait_flag(const int *flag, int *status) {
    long long spins = 0;
    while (*(volatile const int *)flag == 0) {
        if (++spins > kSpinLimit || *(volatile int *)status != 0) {
            atomicExch(status, 1);
            return false;
        }
        __nanosleep(32);
    }
    __threadfence();
    return true;
}

// rows r0 + i (i = lane) of the block: sum over this warp's terms t = warp, warp + 8, ...
// of A[(r0 + i) + (c0 + t) lda] * xs[t] (t < kc), into part[warp][lane]
template <int N>
__device__ __forceinline__ void block_matvec_part(const mlf<N> *A, long long lda, int r0, int kb, int c0, int kc,
                                                  const mlf<N> *xs, mlf<N> (*part)[NB], bool lower_t_le_i,
                                                  bool upper_t_ge_i) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mlf<N> s0 = ml_zero<N>(), s1 = ml_zero<N>();
    if (lane < kb) {
        int q = 0;
        for (int t = warp; t < kc; t += kTrsvWarps, ++q) {
            if (lower_t_le_i && t > lane) continue;
            if (upper_t_ge_i && t < lane) continue;
            const mlf<N> v = ml_mul(A[(r0 + lane) + (long long)(c0 + t) * lda], xs[t]);
            if (q & 1) s1 = ml_add(s1, v);
            else s0 = ml_add(s0, v);
        }
    }
    part[warp][lane] = ml_add(s0, s1);
}

template <int N>
__device__ __forceinline__ mlf<N> sum_parts(mlf<N> (*part)[NB], int lane) {
    const mlf<N> a = ml_add(ml_add(part[0][lane], part[1][lane]), ml_add(part[2][lane], part[3][lane]));
    const mlf<N> b = ml_add(ml_add(part[4][lane], part[5][lane]), ml_add(part[6][lane], part[7][lane]));
    return ml_add(a, b);
}

// backward == 0: x := L^{-1} x (A = L, ld ldl); backward == 1: x := L^{-T} x (A = LT, ld n)
template <int N>
__global__ void __launch_bounds__(kTrsvThreads)
    trsv_wavefront_kernel(int n, const mlf<N> *A, long long lda, const mlf<N> *Dinv, mlf<N> *x, int *sync, int *status,
                          int backward) {
    __shared__ int tk, abort_;
    __shared__ mlf<N> xs[NB];
    __shared__ mlf<N> part[kTrsvWarps][NB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nblk = (n + NB - 1) / NB;
    if (tid == 0) {
        tk = atomicAdd(&sync[0], 1);
        abort_ = 0;
    }
    __syncthreads();
    if (tk >= nblk) return;
    const int b = backward ? nblk - 1 - tk : tk;
    const int r0 = b * NB, kb = min(NB, n - r0);
    mlf<N> acc = ml_zero<N>();  // warp 0, lane i: running sum for row r0 + i
    for (int q = 0; q < tk; ++q) {
        const int c = backward ? nblk - 1 - q : q;
        const int c0 = c * NB, kc = min(NB, n - c0);
        if (tid == 0 && !wait_flag(&sync[1 + c], status)) abort_ = 1;
        __syncthreads();
        if (abort_) return;
        if (tid < kc) xs[tid] = ml_load_cg(x + c0 + tid);  // from L2: written by another CTA
        __syncthreads();
        block_matvec_part<N>(A, lda, r0, kb, c0, kc, xs, part, false, false);
        __syncthreads();
        if (warp == 0) acc = ml_add(acc, sum_parts<N>(part, lane));
        __syncthreads();
    }
    if (warp == 0 && lane < kb) xs[lane] = ml_sub(x[r0 + lane], acc);
    __syncthreads();
    // diagonal: y = Dinv_b rhs (forward) or Dinv_b^T rhs (backward); Dinv_b[i][t] at D[i + NB t]
    const mlf<N> *D = Dinv + (long long)b * NB * NB;
    if (backward) {
        // (Dinv^T)[i][t] = D[t + NB i], t >= i: lanes over i read with stride NB (a 32 x 32 block, cached)
        mlf<N> s0 = ml_zero<N>(), s1 = ml_zero<N>();
        if (lane < kb) {
            int q = 0;
            for (int t = warp; t < kb; t += kTrsvWarps, ++q) {
                if (t < lane) continue;
                const mlf<N> v = ml_mul(D[t + NB * lane], xs[t]);
                if (q & 1) s1 = ml_add(s1, v);
                else s0 = ml_add(s0, v);
            }
        }
        part[warp][lane] = ml_add(s0, s1);
    } else {
        block_matvec_part<N>(D, NB, 0, kb, 0, kb, xs, part, true, false);
    }
    __syncthreads();
    if (warp == 0 && lane < kb) x[r0 + lane] = sum_parts<N>(part, lane);
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicExch(&sync[1 + b], 1);
}

// LT (ld n) = L^T for the lower-triangular n x n L (ld ldl): LT[j + i n] = L[i + j ldl], i >= j
template <int N>
__global__ void transpose_lower_kernel(int n, const mlf<N> *L, int ldl, mlf<N> *LT) {
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    if (j0 > i0 + 31) return;  // tile entirely above the diagonal of L: LT entries unused
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int i = i0 + threadIdx.x, j = j0 + r;  // read L[i][j] coalesced along i
        if (i < n && j < n && i >= j) LT[j + (long long)i * n] = L[i + (long long)j * ldl];
    }
}

template <int N>
GemmProblem<N> gemm_nn(int M, int Nn, int K, const mlf<N> &alpha, const mlf<N> *A, long long lda, char ta,
                       const mlf<N> *B, long long ldb, char tb, const mlf<N> &beta, mlf<N> *C, long long ldc) {
    GemmProblem<N> p{};
    p.M = M;
    p.Nn = Nn;
    p.K = K;
    p.batch = 1;
    p.A = operand_A<N>(ta, A, lda, 0);
    p.B = operand_B<N>(tb, B, ldb, 0);
    p.C = C;
    p.ldc = ldc;
    p.sc = 0;
    p.alpha = alpha;
    p.beta = beta;
    p.lower_only = 0;
    return p;
}

}  // namespace

// Left-looking blocked Cholesky with look-ahead.  Panel k (columns k0 = 32k ..) needs
//     A[k0:, k0:k0+kb] -= L[k0:, :k0] L[k0:k0+kb, :k0]^T
// before it is factored.  The part from the columns of panels 0 .. k-2 is one exact
// (residue-path) product on a side stream, issued as soon as panel k-2 is finished, so it
// runs while panel k-1 is factored; only the previous panel's 32 columns are applied on
// the critical path (panel_update_kernel), then the panel kernel factors panel k.  For
// 256-bit factors of at least 128 rows the products read the residues of the finished
// columns, converted once each (crt_cache_*).
template <int N, int C, int R>
void potrf_panels(int n, mlf<N> *A, int lda, int *info, Workspace &ws, cudaStream_t s) {
    SDPG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
    const size_t mark = ws.used;
    int *sync = (int *)ws.carve(2 * sizeof(int));
    mlf<N> *hist = (mlf<N> *)ws.carve((NB * NB + NB) * sizeof(mlf<N>));
    SDPG_CUDA(cudaMemsetAsync(sync, 0, 2 * sizeof(int), s));
    int *err = ws.error ? ws.error : crt_error_word();
    // the test hook that shortens the tensor-core waits shortens the rows' waits too
    const long long budget = g_tc_wait_cycles > 0 ? g_tc_wait_cycles : kPanelWaitCycles;
    const mlf<N> mone = ml_from_int<N>(-1), one = ml_one<N>();
    const bool cached = crt_cache_applies<N>(n);
    CrtCache cache;
    if (cached) cache = crt_cache_init<N>(n, A, lda, ws.carve(crt_cache_bytes(n)), s);
    const int panels = ceil_div(n, NB);
    static bool attr_set = false;  // dynamic shared memory of the update kernel (97 KB at N = 16)
    if (!attr_set) {
        SDPG_CUDA(cudaFuncSetAttribute(panel_update_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)panel_update_smem<N>()));
        attr_set = true;
    }
    cudaStream_t h = nullptr;  // the side stream, forked from s after the set-up above
    if (panels > 2) {
        ws.ensure_side();
        h = ws.side;
        SDPG_CUDA(cudaEventRecord(ws.ev[0], s));
        SDPG_CUDA(cudaStreamWaitEvent(h, ws.ev[0], 0));
    }
    int ticket0 = 0;
    for (int k = 0; k < panels; ++k) {
        const int k0 = k * NB, kb = min(NB, n - k0), rows = n - k0 - kb;
        if (k >= 2) SDPG_CUDA(cudaStreamWaitEvent(s, ws.ev[2 + (k & 1)], 0));  // product of panels < k-1
        if (k >= 1) {
            SDPG_KT_BEGIN(s);
            panel_update_kernel<N><<<dim3(ceil_div(n - k0, 32), ceil_div(kb, kUpdCols)), 32 * kUpdWarps,
                                     panel_update_smem<N>(), s>>>(
                A, lda, n, k0, kb, k0 - NB);
            SDPG_CHECK_LAUNCH_KT("panel_update_kernel", s);
        }
        const int clusters = 1 + ceil_div(rows, C * R);
        SDPG_KT_BEGIN(s);
        panel_factor_kernel<N, C, R><<<clusters * C, PanelShape<C>::threads, 0, s>>>(
            A, lda, k0, kb, rows, info, hist, sync, 2 * k0, ticket0, budget, err);
        SDPG_CHECK_LAUNCH_KT("panel_factor_kernel", s);
        ticket0 += clusters;
        if (k + 2 < panels) {  // panel k + 2's product with the columns of panels 0 .. k
            SDPG_CUDA(cudaEventRecord(ws.ev[1], s));
            SDPG_CUDA(cudaStreamWaitEvent(h, ws.ev[1], 0));
            const int k2 = k0 + 2 * NB, kb2 = min(NB, n - k2), kend = k0 + NB;
            if (cached) {
                crt_cache_put<N>(cache, A, lda, k0, kb, ws.error, h);
                crt_cache_panel<N>(cache, k2, kb2, kend, A, lda, ws.error, h);
            } else {
                GemmProblem<N> p = gemm_nn<N>(n - k2, kb2, kend, mone, A + k2, lda, 'N', A + k2, lda, 'T', one,
                                              A + k2 + (long long)k2 * lda, lda);
                p.lower_only = 1;
                const size_t m2 = ws.used;
                ml_gemm<N>(p, ws, h);
                ws.used = m2;
            }
            SDPG_CUDA(cudaEventRecord(ws.ev[2 + ((k + 2) & 1)], h));
        }
    }
    if (h) {  // join
        SDPG_CUDA(cudaEventRecord(ws.ev[1], h));
        SDPG_CUDA(cudaStreamWaitEvent(s, ws.ev[1], 0));
    }
    ws.used = mark;
}

template <int N>
void ml_potrf(int n, mlf<N> *A, int lda, int *info, Workspace &ws, cudaStream_t s) {
    static_assert(kPanelRowWarps * 32 <= PanelShape<kPanelCluster>::threads, "one row per warp");
    potrf_panels<N, kPanelCluster, kPanelRowWarps>(n, A, lda, info, ws, s);
}

template <int N>
size_t ml_potrf_workspace_bytes(int n) {
    GemmProblem<N> p{};
    p.M = n;
    p.Nn = NB;
    p.K = n;
    p.batch = 1;
    size_t b = gemm_workspace_bytes<N>(p);
    if (crt_cache_applies<N>(n)) b = std::max(b, crt_cache_bytes(n));
    return b + (size_t)(NB + NB * NB) * sizeof(mlf<N>) + 4096;  // history, progress words, alignment
}

namespace {

template <int N>
__global__ void pad_lower_kernel(int n, int P, const mlf<N> *L, int ldl, mlf<N> *Lp) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)P * P) return;
    const int i = (int)(q % P), j = (int)(q / P);
    mlf<N> v = ml_zero<N>();
    if (i < n && j < n) {
        if (i >= j) v = L[i + (long long)j * ldl];
    } else if (i == j) {
        v = ml_one<N>();
    }
    Lp[q] = v;
}

template <int N>
__global__ void unpad_kernel(int n, int P, const mlf<N> *Xp, mlf<N> *X) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)n * n) return;
    const int i = (int)(q % n), j = (int)(q / n);
    X[q] = Xp[i + (long long)j * P];
}

inline int trtri_pad(int n) {
    int P = NB;
    while (P < n) P *= 2;
    return P;
}

}  // namespace

template <int N>
size_t ml_trtri_workspace_bytes(int n) {
    const int P = trtri_pad(n);
    const size_t pp = (size_t)P * P;
    GemmProblem<N> g{};
    g.M = P / 2;
    g.Nn = P / 2;
    g.K = P / 2;
    g.batch = 1;
    // padded L and X, the per-level W, and the scratch of the top level's GEMM (a level with
    // node size b quantises P*b/4 entries per operand, so the top level is the largest),
    // with slack for alignment
    return 2 * pp * sizeof(mlf<N>) + pp / 2 * sizeof(mlf<N>) + 2 * gemm_workspace_bytes<N>(g) + (64u << 10);
}

// Linv = L^{-1}: pad L to P = 32 * 2^k with an identity tail, invert the 32 x 32 diagonal
// blocks in parallel, then for node sizes b = 64, 128, ..., P form every node's
// off-diagonal block X21 = -X22 (L21 X11) with one batched GEMM pair per level.
template <int N>
void ml_trtri_lower(int n, const mlf<N> *L, int ldl, mlf<N> *Linv, Workspace &ws, cudaStream_t s) {
    const int P = trtri_pad(n);
    const size_t mark = ws.used;
    const long long pp = (long long)P * P;
    mlf<N> *Lp = (mlf<N> *)ws.carve(pp * sizeof(mlf<N>));
    mlf<N> *Xp = (mlf<N> *)ws.carve(pp * sizeof(mlf<N>));
    mlf<N> *W = (mlf<N> *)ws.carve(pp / 2 * sizeof(mlf<N>));
    SDPG_KT_BEGIN(s);
    pad_lower_kernel<N><<<ceil_div(pp, 256), 256, 0, s>>>(n, P, L, ldl, Lp);
    SDPG_CHECK_LAUNCH_KT("pad_lower_kernel", s);
    SDPG_CUDA(cudaMemsetAsync(Xp, 0, pp * sizeof(mlf<N>), s));
    SDPG_KT_BEGIN(s);
    trtri_diag_kernel<N><<<(P / NB) * kPanelCluster, PanelShape<kPanelCluster>::threads, 0, s>>>(
        Lp, P, Xp, P, ws.error ? ws.error : crt_error_word());
    SDPG_CHECK_LAUNCH_KT("trtri_diag_kernel", s);
    const mlf<N> one = ml_one<N>(), zero = ml_zero<N>(), mone = ml_from_int<N>(-1);
    for (int b = 2 * NB; b <= P; b *= 2) {
        const int h = b / 2, nodes = P / b;
        const long long node_stride = (long long)b * (1 + P);
        // W_t = L21 X11  (h x h x h), batched over nodes
        GemmProblem<N> p{};
        p.M = h;
        p.Nn = h;
        p.K = h;
        p.batch = nodes;
        p.A = operand_A<N>('N', Lp + h, P, node_stride);
        p.B = operand_B<N>('N', Xp, P, node_stride);
        p.C = W;
        p.ldc = h;
        p.sc = (long long)h * h;
        p.alpha = one;
        p.beta = zero;
        p.lower_only = 0;
        {
            const size_t m2 = ws.used;
            ml_gemm<N>(p, ws, s);
            ws.used = m2;
        }
        // X21 = -X22 W_t
        p.A = operand_A<N>('N', Xp + h + (long long)h * P, P, node_stride);
        p.B = operand_B<N>('N', W, h, (long long)h * h);
        p.C = Xp + h;
        p.ldc = P;
        p.sc = node_stride;
        p.alpha = mone;
        {
            const size_t m2 = ws.used;
            ml_gemm<N>(p, ws, s);
            ws.used = m2;
        }
    }
    SDPG_KT_BEGIN(s);
    unpad_kernel<N><<<ceil_div((long long)n * n, 256), 256, 0, s>>>(n, P, Xp, Linv);
    SDPG_CHECK_LAUNCH_KT("unpad_kernel", s);
    ws.used = mark;
}

// prepared data: the packed inverted diagonal blocks, the transposed factor (ld n),
// then the wavefront synchronisation words and a status word
template <int N>
size_t ml_potrs_prepare_bytes(int n) {
    const size_t nblk = ceil_div(n, NB);
    return (nblk * NB * NB + (size_t)n * n) * sizeof(mlf<N>) + (2 * (nblk + 1) + 1) * sizeof(int) + 256;
}

template <int N>
void ml_potrs_prepare(int n, const mlf<N> *L, int ldl, mlf<N> *Dinv, cudaStream_t s) {
    SDPG_KT_BEGIN(s);
    trtri_diag_packed_kernel<N><<<ceil_div(n, NB), 256, 0, s>>>(L, ldl, Dinv, n);
    SDPG_CHECK_LAUNCH_KT("trtri_diag_packed_kernel", s);
    mlf<N> *LT = Dinv + (size_t)ceil_div(n, NB) * NB * NB;
    SDPG_KT_BEGIN(s);
    transpose_lower_kernel<N><<<dim3(ceil_div(n, 32), ceil_div(n, 32)), dim3(32, 8), 0, s>>>(n, L, ldl, LT);
    SDPG_CHECK_LAUNCH_KT("transpose_lower_kernel", s);
}

template <int N>
void ml_potrs_solve(int n, const mlf<N> *L, int ldl, const mlf<N> *Dinv, mlf<N> *x, cudaStream_t s) {
    const int nblk = ceil_div(n, NB);
    const mlf<N> *LT = Dinv + (size_t)nblk * NB * NB;
    int *sync = (int *)(((uintptr_t)(LT + (size_t)n * n) + 255) & ~(uintptr_t)255);
    int *status = sync + 2 * (nblk + 1);
    SDPG_CUDA(cudaMemsetAsync(sync, 0, (2 * (nblk + 1) + 1) * sizeof(int), s));
    SDPG_KT_BEGIN(s);
    trsv_wavefront_kernel<N><<<nblk, kTrsvThreads, 0, s>>>(n, L, ldl, Dinv, x, sync, status, 0);
    SDPG_CHECK_LAUNCH_KT("trsv_wavefront_kernel", s);
    SDPG_KT_BEGIN(s);
    trsv_wavefront_kernel<N><<<nblk, kTrsvThreads, 0, s>>>(n, LT, n, Dinv, x, sync + nblk + 1, status, 1);
    SDPG_CHECK_LAUNCH_KT("trsv_wavefront_kernel", s);
}

template <int N>
int *ml_potrs_status(int n, mlf<N> *Dinv) {
    const int nblk = ceil_div(n, NB);
    const mlf<N> *LT = Dinv + (size_t)nblk * NB * NB;
    int *sync = (int *)(((uintptr_t)(LT + (size_t)n * n) + 255) & ~(uintptr_t)255);
    return sync + 2 * (nblk + 1);
}

template <int N>
void ml_potrs(int n, const mlf<N> *L, int ldl, mlf<N> *x, Workspace &ws, cudaStream_t s) {
    const size_t mark = ws.used;
    mlf<N> *Dinv = (mlf<N> *)ws.carve(ml_potrs_prepare_bytes<N>(n));
    ml_potrs_prepare<N>(n, L, ldl, Dinv, s);
    ml_potrs_solve<N>(n, L, ldl, Dinv, x, s);
    ws.used = mark;
}

#define SDPG_INST_CHOL(N)                                                                       \
    template void ml_potrf<N>(int, mlf<N> *, int, int *, Workspace &, cudaStream_t);            \
    template size_t ml_potrf_workspace_bytes<N>(int);                                                       \
    template void ml_trtri_lower<N>(int, const mlf<N> *, int, mlf<N> *, Workspace &, cudaStream_t); \
    template size_t ml_trtri_workspace_bytes<N>(int);                                                       \
    template void ml_potrs<N>(int, const mlf<N> *, int, mlf<N> *, Workspace &, cudaStream_t);             \
    template size_t ml_potrs_prepare_bytes<N>(int);                                                        \
    template void ml_potrs_prepare<N>(int, const mlf<N> *, int, mlf<N> *, cudaStream_t);                    \
    template void ml_potrs_solve<N>(int, const mlf<N> *, int, const mlf<N> *, mlf<N> *, cudaStream_t);        \
    template int *ml_potrs_status<N>(int, mlf<N> *);
SDPG_INST_CHOL(8)
SDPG_INST_CHOL(16)

}  // namespace sdpg
