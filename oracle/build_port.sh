#!/usr/bin/env bash
# Build the CPU port of the reference solver (oracle/sdpa_port.cpp) into
# oracle/_port/ -- test infrastructure only (timed CPU baseline and checker).
# Links the system GMP runtime by path (no GMP development files needed).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
GMPLIB=""
for cand in /usr/lib/x86_64-linux-gnu/libgmp.so.10 /usr/lib/aarch64-linux-gnu/libgmp.so.10 \
            /usr/lib64/libgmp.so.10 /usr/lib/libgmp.so.10; do
    if [ -f "$cand" ]; then GMPLIB="$cand"; break; fi
done
if [ -z "$GMPLIB" ]; then
    echo "build_port: libgmp.so.10 not found" >&2
    exit 2
fi
mkdir -p "$HERE/_port"
if [ ! -x "$HERE/_port/sdpa_port" ] || [ "$HERE/sdpa_port.cpp" -nt "$HERE/_port/sdpa_port" ] \
   || [ "$HERE/gmp_abi.h" -nt "$HERE/_port/sdpa_port" ]; then
    g++ -O2 -fopenmp -std=c++17 -o "$HERE/_port/sdpa_port" "$HERE/sdpa_port.cpp" "$GMPLIB"
fi
echo "$HERE/_port/sdpa_port"
