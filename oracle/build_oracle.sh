#!/usr/bin/env bash
# Builds oracle/libnr_oracle.so from nr_oracle.c.  -ffp-contract=off keeps
# the compiler from fusing multiply-adds (every fma in the oracle is an
# explicit fma()); on x86-64 hosts with FMA units -mfma lets fma() inline
# (same correctly rounded result, no libm call).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
CC="${CC:-gcc}"
EXTRA=""
if [ "$(uname -m)" = "x86_64" ] && grep -qw fma /proc/cpuinfo 2>/dev/null; then
    EXTRA="-mfma"
fi
"$CC" -std=c11 -O2 -fPIC -shared -ffp-contract=off $EXTRA -o "$HERE/libnr_oracle.so.tmp" "$HERE/nr_oracle.c" "$HERE/nr_oracle_mesh.c" "$HERE/nr_oracle_spr.c" -lm -lpthread
mv "$HERE/libnr_oracle.so.tmp" "$HERE/libnr_oracle.so"
