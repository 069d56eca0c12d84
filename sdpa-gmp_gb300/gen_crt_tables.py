"""Generate csrc/crt_tables.h: the constants of the residue-number-system GEMM path.

For a K-term sum of products of integers below 2^R (R = 276 for 256-bit operands,
K <= 1024), |V| < 2^562; the moduli are the largest primes below 512 whose product
M exceeds 2^568, so V / M lies well inside (-1/2, 1/2).  Per modulus m:
  cfac  = (M / m)^-1 mod m                  (CRT factor applied in the GEMM epilogue)
  pow16 = 2^(16 c) mod m, c = 0 .. 17        (residue of a 288-bit integer from 16-bit chunks)
  inv   = floor(2^320 cfac / m) as ten 32-bit words: with r_l = V mod m_l,
          V / M = sum_l r_l cfac_l / m_l (mod 1), so the tensor-core epilogue stores r_l
          and the CRT factor is folded into this table
and M itself as a 256-bit mantissa with its exponent.

Run: python sdpa-gmp_gb300/gen_crt_tables.py  (writes the header beside the sources)
"""
import os


def primes_below(n):
    sieve = [True] * n
    sieve[0] = sieve[1] = False
    for i in range(2, int(n ** 0.5) + 1):
        if sieve[i]:
            for j in range(i * i, n, i):
                sieve[j] = False
    return [i for i in range(n) if sieve[i]]


def main():
    moduli, prod = [], 1
    for p in reversed(primes_below(512)):
        moduli.append(p)
        prod *= p
        if prod.bit_length() > 568:
            break
    L = len(moduli)
    cfac = [pow(prod // m, -1, m) for m in moduli]
    pow16 = [[pow(2, 16 * c, m) for c in range(18)] for m in moduli]
    inv = [(c << 320) // m for c, m in zip(cfac, moduli)]
    inv_words = [[(v >> (32 * w)) & 0xFFFFFFFF for w in range(10)] for v in inv]
    bl = prod.bit_length()
    mant = prod >> (bl - 256)  # top 256 bits (truncated)
    mant_words = [(mant >> (32 * w)) & 0xFFFFFFFF for w in range(8)]
    out = []
    out.append("// Generated by gen_crt_tables.py -- constants of the residue-number-system GEMM.")
    out.append("#pragma once")
    out.append("#include <stdint.h>")
    out.append("namespace sdpg {")
    out.append(f"constexpr int kCrtL = {L};              // moduli")
    out.append("constexpr int kCrtR = 276;             // bits of the integer operands")
    out.append("constexpr int kCrtInvWords = 10;       // 2^320 cfac / m as 32-bit words")
    out.append("constexpr int kCrtPowChunks = 18;      // 16-bit chunks of a 288-bit integer")
    out.append(f"constexpr int kCrtMtotExp = {bl};       // M = 0.mant * 2^kCrtMtotExp")
    out.append("static const int kCrtModuli[kCrtL] = {" + ", ".join(map(str, moduli)) + "};")
    out.append("static const int kCrtCfac[kCrtL] = {" + ", ".join(map(str, cfac)) + "};")
    out.append("static const int kCrtPow16[kCrtL][kCrtPowChunks] = {")
    for row in pow16:
        out.append("    {" + ", ".join(map(str, row)) + "},")
    out.append("};")
    out.append("static const uint32_t kCrtInv[kCrtL][kCrtInvWords] = {")
    for row in inv_words:
        out.append("    {" + ", ".join(f"0x{w:08x}u" for w in row) + "},")
    out.append("};")
    out.append("static const uint32_t kCrtMtotMant[8] = {" + ", ".join(f"0x{w:08x}u" for w in mant_words) + "};")
    out.append("}  // namespace sdpg")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "crt_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print(f"wrote {path}: {L} moduli, M has {bl} bits")


if __name__ == "__main__":
    main()
