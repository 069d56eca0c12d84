// Exact modular GEMMs on the fifth-generation tensor cores (tcgen05).
//
// Used by the residue-number-system (Chinese remainder) path of the multi-limb GEMM:
// every operand entry is an integer held as its residues modulo L small primes
// m_l < 512, stored as fp16 in the balanced range [-(m_l-1)/2, (m_l-1)/2].  For each
// modulus the kernel forms S = A_l B_l^T with fp16 products accumulated in fp32 in
// tensor memory.  Every partial sum is an integer of magnitude at most
// 256 * 255^2 < 2^24 when at most 256 products are summed, so the fp32 accumulation
// is exact; longer K is split over up to four accumulators of 256 each.  The
// epilogue writes y_l = S mod m_l (the CRT factor lives in the reconstruction table).
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace sdpg {

constexpr int kTcBM = 128;      // tile rows (tcgen05 M)
constexpr int kTcBN = 128;      // tile columns (tcgen05 N)
constexpr int kTcBK = 64;       // K block: one 128-byte swizzle row of fp16
constexpr int kTcKChunk = 256;  // products per exact fp32 accumulator
constexpr int kTcMaxK = 1024;   // four accumulators of 128 columns fill tensor memory

struct TcModGemm {
    const __half *A;  // planes [zA][Mpad][Kpad], K contiguous
    const __half *B;  // planes [zB][Npad][Kpad], K contiguous
    uint16_t *Y;      // planes [z][Mpad][Npad]: S mod m_l
    int L;            // moduli
    int batch;        // z = b * L + l; A plane (bA * L + l) with bA = b if a_batched else 0
    int a_batched, b_batched;
    int Mpad, Npad, Kpad;  // multiples of 128, 128, 64; Kpad <= kTcMaxK: the K range of this call
    int a_rows, b_rows;    // rows between consecutive planes of A / B (0: Mpad / Npad); the
                           // Y planes are always Mpad x Npad
    int a_skip, b_skip;    // rows of the first plane before A / B (the pointers sit that far
                           // into a plane store whose planes are a_rows / b_rows apart)
    int k0;                // first K index of this call within the planes (a multiple of 64)
    int kpitch;            // K extent of the planes (their row length)
    int kext;              // columns the maps may read (0: kpitch); from kext on they read as zero
    int accumulate;        // 1: Y = (Y + new) mod m (a later K chunk of the same product)
    int lower_only;        // 1: skip tiles strictly above the diagonal (their Y is not written)
    const int *moduli;     // device, L entries
    int *error;            // device word of the caller: set non-zero if a bounded wait timed out
    int *sticky;           // device-wide flag, also set (may equal error or be null)
    long long wait_cycles; // budget of the producer's and MMA issuer's waits (set by tc_modgemm)
    double alg_flops;      // algorithmic fp16 flops of this call (per-kernel timing only)
};

// Budget in clock cycles of the tensor-core kernel's primary waits (TMA data, free
// stages); 0 = the default of about one second.  Shortening it is a test hook that makes
// those waits give up; the drains after a give-up keep the full budget.
extern long long g_tc_wait_cycles;

// Y planes for all (b, l); grid (Npad/128, Mpad/128, batch*L), 128 threads, one tile each.
void tc_modgemm(const TcModGemm &p, cudaStream_t s);

}  // namespace sdpg
