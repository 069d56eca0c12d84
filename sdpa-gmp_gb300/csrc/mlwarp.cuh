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

// ---- exact sums in signed fixed point ----
// A group of values is summed as two's-complement integers of W = N + 2 words relative to
// the group's largest exponent E (a value of exponent E has its mantissa in words 1..N,
// the top word is headroom and sign), so the tree needs only word-wise integer adds and
// the sum is rounded to N limbs once.  Each value loses the bits below 2^-32 of the
// frame's last mantissa word, about 2^-(32N+32) of the largest value.
constexpr int kFixNone = -(1 << 30);  // exponent of a group with no nonzero value

template <int N>
MLHD void ml_to_fix(const mlf<N> &v, int E, uint32_t (&a)[N + 2]) {
    constexpr int W = N + 2;
    a[0] = 0u;
    ML_UNROLL
    for (int k = 0; k < N; ++k) a[k + 1] = v.m[k];
    a[N + 1] = 0u;
    const int delta = E - v.e;
    const bool zero = v.m[N - 1] == 0u || delta >= 32 * W || delta < 0;
    ml_limb_shr<W>(a, zero ? 0 : (delta >> 5));
    ml_bit_shr<W>(a, zero ? 0 : (delta & 31));
    uint32_t carry = v.s ? 1u : 0u;  // negative: ~a + 1
    ML_UNROLL
    for (int k = 0; k < W; ++k) {
        const uint32_t x = zero ? 0u : (v.s ? ~a[k] : a[k]);
        const uint64_t t = (uint64_t)x + (zero ? 0u : carry);
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
}

template <int W>
MLHD void ml_fix_add(uint32_t (&a)[W], const uint32_t (&b)[W]) {
    uint32_t carry = 0u;
    ML_UNROLL
    for (int k = 0; k < W; ++k) {
        const uint64_t t = (uint64_t)a[k] + b[k] + carry;
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
}

// the fixed-point sum of a group with largest exponent E, rounded to N limbs
template <int N>
MLHD mlf<N> ml_from_fix(uint32_t (&a)[N + 2], int E) {
    constexpr int W = N + 2;
    if (E == kFixNone) return ml_zero<N>();
    const bool neg = (a[W - 1] >> 31) != 0u;
    uint32_t carry = 1u;
    ML_UNROLL
    for (int k = 0; k < W; ++k) {  // |a|
        const uint64_t t = (uint64_t)(neg ? ~a[k] : a[k]) + (neg ? carry : 0u);
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
    return ml_pack<N, W>(a, E + 32, neg ? 1u : 0u);
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
