// Warp / block level helpers for mlf values (device only).
#pragma once
#include "ml.cuh"
#include "mlfix.cuh"

namespace sdpg {

template <int N>
__device__ __forceinline__ mlf<N> ml_shfl_xor(const mlf<N> &v, int off) {
    mlf<N> r;
    r.e = __shfl_xor_sync(0xffffffffu, v.e, off);
    r.s = __shfl_xor_sync(0xffffffffu, v.s, off);
#pragma unroll
    for (int k = 0; k < N; ++k) r.m[k] = __shfl_xor_sync(0xffffffffu, v.m[k], off);
    return r;
}

template <int N>
__device__ __forceinline__ mlf<N> ml_shfl(const mlf<N> &v, int src) {
    mlf<N> r;
    r.e = __shfl_sync(0xffffffffu, v.e, src);
    r.s = __shfl_sync(0xffffffffu, v.s, src);
#pragma unroll
    for (int k = 0; k < N; ++k) r.m[k] = __shfl_sync(0xffffffffu, v.m[k], src);
    return r;
}

__device__ __forceinline__ int warp_max_int(int e) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
    return e;
}

template <int W>
__device__ __forceinline__ void fix_warp_tree(uint32_t (&a)[W]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        uint32_t b[W];
#pragma unroll
        for (int k = 0; k < W; ++k) b[k] = __shfl_xor_sync(0xffffffffu, a[k], off);
        ml_fix_add<W>(a, b);
    }
}

// Sum over the 32 lanes, exact up to the fixed-point frame, rounded once; every lane
// returns it.
template <int N>
__device__ __forceinline__ mlf<N> ml_warp_sum(mlf<N> v) {
    const int E = warp_max_int(v.m[N - 1] ? v.e : kFixNone);
    uint32_t a[N + 2];
    ml_to_fix<N>(v, E, a);
    fix_warp_tree<N + 2>(a);
    return ml_from_fix<N>(a, E);
}

template <int N>
__device__ __forceinline__ mlf<N> ml_warp_maxabs(mlf<N> v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const mlf<N> o = ml_shfl_xor(v, off);
        if (ml_cmp_abs(o, v) > 0) v = o;
    }
    return v;
}

// Out-of-line multi-limb operations for the latency-bound control kernels (one CTA or
// one warp running a long dependent chain: the Lanczos update and loop control, the
// tridiagonal eigenvalue).  Fully inlined, their straight-line bodies outgrow the
// instruction cache and the warps stall on instruction fetch; called, one copy of each
// stays resident.  Arguments and results travel in registers.
template <int N>
__device__ __noinline__ mlf<N> mlc_add(mlf<N> a, mlf<N> b) { return ml_add(a, b); }
template <int N>
__device__ __noinline__ mlf<N> mlc_sub(mlf<N> a, mlf<N> b) { return ml_sub(a, b); }
template <int N>
__device__ __noinline__ mlf<N> mlc_mul(mlf<N> a, mlf<N> b) { return ml_mul(a, b); }
template <int N>
__device__ __noinline__ mlf<N> mlc_div(mlf<N> a, mlf<N> b) { return ml_div(a, b); }
template <int N>
__device__ __noinline__ mlf<N> mlc_rsqrt(mlf<N> a) { return ml_rsqrt(a); }

// Block sum (blockDim.x a multiple of 32, <= 1024) in one fixed-point frame for the whole
// block: exact up to the frame, rounded once; result valid on thread 0 (on all of warp 0).
template <int N>
__device__ __forceinline__ mlf<N> ml_block_sum(mlf<N> v) {
    constexpr int W = N + 2;
    __shared__ int emax[32];
    __shared__ uint32_t part[32][W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    int E = warp_max_int(v.m[N - 1] ? v.e : kFixNone);
    if (lane == 0) emax[warp] = E;
    __syncthreads();
    E = kFixNone;
    for (int w = 0; w < nw; ++w) E = max(E, emax[w]);
    uint32_t a[W];
    ml_to_fix<N>(v, E, a);
    fix_warp_tree<W>(a);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < W; ++k) part[warp][k] = a[k];
    }
    __syncthreads();
    mlf<N> r = ml_zero<N>();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < W; ++k) a[k] = lane < nw ? part[lane][k] : 0u;
        fix_warp_tree<W>(a);
        r = ml_from_fix<N>(a, E);
    }
    __syncthreads();
    return r;
}

// The same names for the control kernels (the fixed-point sums are short enough inline).
template <int N>
__device__ __forceinline__ mlf<N> mlc_warp_sum(mlf<N> v) {
    return ml_warp_sum<N>(v);
}
template <int N>
__device__ __forceinline__ mlf<N> mlc_block_sum(mlf<N> v) {
    return ml_block_sum<N>(v);
}

template <int N>
__device__ __forceinline__ mlf<N> ml_block_maxabs(mlf<N> v) {
    __shared__ mlf<N> part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = ml_warp_maxabs(v);
    if (lane == 0) part[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        v = lane < nw ? part[lane] : ml_zero<N>();
        v = ml_warp_maxabs(v);
    }
    __syncthreads();
    return v;
}

}  // namespace sdpg
