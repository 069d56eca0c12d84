#!/usr/bin/env bash
# Build the unmodified reference solver (sdpa_gmp) from its own sources into
# oracle/_ref/ — test infrastructure only (it is the parity oracle and the
# timed CPU reference, never part of the product).
#
# Recipe (no reference build system is run):
#   * the source list is read from the reference's Makefile.am (the
#     non-SYSTEM_MPLAPACK branch, Makefile.am:11-49);
#   * gmp.h is generated from the vendored GMP 6.2.1 template gmp-h.in by
#     substituting its @VAR@ placeholders for a 64-bit-limb LP64 host;
#     gmpxx.h is taken from the same tarball; both land in oracle/_ref/include;
#   * the runtime library is the system libgmp.so.10 (GMP 6.3.0 runtime, same
#     ABI), linked by full path because no development symlink is installed;
#   * the missing SPOOLES headers are replaced by oracle/spooles_shim.h and its
#     entry points by abort stubs (never reached for nBlock <= 5);
#   * libgmpxx's stream inserters come from oracle/gmpxx_streams.cpp.
# Flags follow Makefile.am:56 (-O2 -fopenmp -DUseMETIS=0) minus -march=native.
#
# Usage: oracle/build_ref.sh [REFERENCE_DIR]
#   (default: $SDPG_REFERENCE_DIR, else /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${SDPG_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/sdpa_main.cpp" ]; then
    echo "build_ref: reference sources not found at $REF" >&2
    exit 2
fi
GMPLIB=""
for cand in /usr/lib/x86_64-linux-gnu/libgmp.so.10 /usr/lib/aarch64-linux-gnu/libgmp.so.10 \
            /usr/lib64/libgmp.so.10 /usr/lib/libgmp.so.10; do
    if [ -f "$cand" ]; then GMPLIB="$cand"; break; fi
done
if [ -z "$GMPLIB" ]; then
    echo "build_ref: libgmp.so.10 not found" >&2
    exit 2
fi
mkdir -p "$OUT/include" "$OUT/obj"
TARBALL="$REF/external/gmp/download/gmp-6.2.1.tar.bz2"
tar -xjf "$TARBALL" -O gmp-6.2.1/gmp-h.in | sed \
    -e 's/@HAVE_HOST_CPU_FAMILY_power@/0/' \
    -e 's/@HAVE_HOST_CPU_FAMILY_powerpc@/0/' \
    -e 's/@GMP_LIMB_BITS@/64/' \
    -e 's/@GMP_NAIL_BITS@/0/' \
    -e 's/@DEFN_LONG_LONG_LIMB@//' \
    -e 's/@LIBGMP_DLL@/0/' \
    -e 's/@CC@/gcc/' \
    -e 's/@CFLAGS@/-O2/' > "$OUT/include/gmp.h"
tar -xjf "$TARBALL" -O gmp-6.2.1/gmpxx.h > "$OUT/include/gmpxx.h"
for h in InpMtx IVL Graph ETree misc IV SymbFac; do
    echo '#include "spooles_shim.h"' > "$OUT/include/$h.h"
done

# Sources of the non-system-MPLAPACK branch of Makefile.am.
SRCS=$(awk '/^else/{f=1;next} /^endif/{f=0} f' "$REF/Makefile.am" | tr -d '\\' | tr ' \t' '\n\n' | grep '\.cpp$' | sort -u)
CXXFLAGS="-O2 -fopenmp -DUseMETIS=0 -w -I$OUT/include -I$HERE -I$REF -I$REF/mplapack"
JOBS=$(nproc 2>/dev/null || echo 4)
OBJS=()
pids=()
for s in $SRCS; do
    o="$OUT/obj/$(echo "$s" | tr '/' '_' | sed 's/\.cpp$/.o/')"
    OBJS+=("$o")
    if [ ! -f "$o" ] || [ "$REF/$s" -nt "$o" ]; then
        g++ $CXXFLAGS -c "$REF/$s" -o "$o" &
        pids+=($!)
        if [ "${#pids[@]}" -ge "$JOBS" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
    fi
done
for p in "${pids[@]}"; do wait "$p"; done
gcc -O2 -c "$HERE/spooles_stubs.c" -I"$HERE" -o "$OUT/obj/spooles_stubs.o"
g++ $CXXFLAGS -c "$HERE/gmpxx_streams.cpp" -o "$OUT/obj/gmpxx_streams.o"
g++ -fopenmp -o "$OUT/sdpa_gmp" "${OBJS[@]}" "$OUT/obj/spooles_stubs.o" "$OUT/obj/gmpxx_streams.o" "$GMPLIB"
echo "build_ref: built $OUT/sdpa_gmp"
