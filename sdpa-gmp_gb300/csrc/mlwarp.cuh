// Warp / block level helpers for mlf values (device only).
#pragma once
#include "ml.cuh"

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

// Sum over the 32 lanes; the value returned on lane 0 is the one to use.
template <int N>
__device__ __forceinline__ mlf<N> ml_warp_sum(mlf<N> v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = ml_add(v, ml_shfl_xor(v, off));
    return v;
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

template <int N>
__device__ __forceinline__ mlf<N> mlc_warp_sum(mlf<N> v) {
#pragma unroll 1
    for (int off = 16; off > 0; off >>= 1) v = mlc_add(v, ml_shfl_xor(v, off));
    return v;
}

// Block sum with the out-of-line addition; result valid on thread 0.
template <int N>
__device__ __forceinline__ mlf<N> mlc_block_sum(mlf<N> v) {
    __shared__ mlf<N> part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = mlc_warp_sum(v);
    if (lane == 0) part[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        v = lane < nw ? part[lane] : ml_zero<N>();
        v = mlc_warp_sum(v);
    }
    __syncthreads();
    return v;
}

// Block sum (blockDim.x a multiple of 32, <= 1024); result valid on thread 0.
template <int N>
__device__ __forceinline__ mlf<N> ml_block_sum(mlf<N> v) {
    __shared__ mlf<N> part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = ml_warp_sum(v);
    if (lane == 0) part[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        v = lane < nw ? part[lane] : ml_zero<N>();
        v = ml_warp_sum(v);
    }
    __syncthreads();
    return v;
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
