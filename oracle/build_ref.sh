#!/usr/bin/env bash
# Builds oracle/_ref/liblsr_ref.so and oracle/_ref/libnmr_ref.so: the
# reference's own large_strain_relax.cu and network_mesh_relax.cu compiled as
# host C++ (kernels run as sequential loops, cuBLAS Level-1 and the CUDA
# runtime replaced by the stand-ins in oracle/refshim/include); and
# oracle/_ref/libspr_ref.so: sparse_relax.cpp, unchanged, against the dense
# CHOLMOD / SPQR stand-ins of oracle/refshim/spr_include (SuiteSparse and
# MKL are not in this image); the analysis programs strain_calc and
# axial_contribution as executables; and oracle/_ref/libna_ref.so:
# na_calc.cpp against the std stand-ins of oracle/refshim/boost_include.
#
# The source is read where it lies and piped to the compiler with two textual
# rewrites.  The first is the kernel-launch syntax, `k<<<grid, block>>>(args)`
# -> `nr_ref_launch(grid, block, k, args)`, which plain C++ cannot parse.
# The second is the one-token fix at large_strain_relax.cu:349 and
# network_mesh_relax.cu:465, `mass < 0 || fcut < 0 || nmax < 0` compares
# pointers with 0, which GCC 13 rejects; the parsed values `*mass`, `*fcut`,
# `*nmax` are what it means.
# main is renamed so the library can expose the CLI.
#
# Needs the reference checkout (default /root/reference, or $NR_REFERENCE).
# Outputs go only to oracle/_ref/ (git-ignored).  Exits 0 without building
# when the reference is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${NR_REFERENCE:-/root/reference}"
SRC="$REF/src/large_strain_relax.cu"
MESH_SRC="$REF/src/network_mesh_relax.cu"
OUT="$HERE/_ref"
if [ ! -f "$SRC" ]; then
    echo "build_ref: $SRC not present; skipping"
    exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
host_compile() { # <source> <renamed main> <object>
    sed -E -e 's/([A-Za-z_][A-Za-z0-9_]*)<<<([^>]*)>>>\(/nr_ref_launch(\2, \1, /g' \
        -e 's/\|\| mass < 0 \|\| fcut < 0 \|\| nmax < 0/|| *mass < 0 || *fcut < 0 || *nmax < 0/' "$1" |
        "$CXX" -x c++ -std=c++17 -O2 -fPIC -w \
            -I "$HERE/refshim/include" -I "$REF/src" -Dmain="$2" \
            -c - -o "$3"
}
shim() { "$CXX" -std=c++17 -O2 -fPIC -I "$HERE/refshim/include" -c "$HERE/refshim/$1.cpp" -o "$OUT/$1.o"; }
shim shim_common
host_compile "$SRC" lsr_reference_main "$OUT/lsr_ref.o"
shim ref_api
"$CXX" -shared -o "$OUT/liblsr_ref.so" "$OUT/lsr_ref.o" "$OUT/ref_api.o" "$OUT/shim_common.o"
echo "build_ref: built $OUT/liblsr_ref.so"
if [ -f "$REF/src/sparse_relax.cpp" ]; then
    "$CXX" -x c++ -std=c++17 -O2 -fPIC -w -I "$HERE/refshim/spr_include" -I "$REF/src" \
        -Dmain=spr_reference_main -c "$REF/src/sparse_relax.cpp" -o "$OUT/spr_ref.o"
    "$CXX" -std=c++17 -O2 -fPIC -I "$HERE/refshim/spr_include" -c "$HERE/refshim/ref_spr_api.cpp" \
        -o "$OUT/ref_spr_api.o"
    "$CXX" -shared -o "$OUT/libspr_ref.so" "$OUT/spr_ref.o" "$OUT/ref_spr_api.o" "$OUT/shim_common.o"
    echo "build_ref: built $OUT/libspr_ref.so"
fi
if [ -f "$MESH_SRC" ]; then
    host_compile "$MESH_SRC" nmr_reference_main "$OUT/nmr_ref.o"
    shim ref_mesh_api
    "$CXX" -shared -o "$OUT/libnmr_ref.so" "$OUT/nmr_ref.o" "$OUT/ref_mesh_api.o" "$OUT/shim_common.o"
    echo "build_ref: built $OUT/libnmr_ref.so"
fi
# The analysis programs strain_calc.cpp and axial_contribution.cpp need only
# the standard library: built unchanged as executables.
for prog in strain_calc axial_contribution; do
    if "$CXX" -std=c++17 -O2 -w "$REF/src/$prog.cpp" -o "$OUT/$prog"; then
        echo "build_ref: built $OUT/$prog"
    else
        echo "build_ref: $prog not built"
    fi
done
# na_calc.cpp includes Boost.Filesystem and Boost.Regex, which are absent:
# it is compiled unchanged against the std::filesystem / std::regex
# stand-ins of oracle/refshim/boost_include, with main renamed, into
# oracle/_ref/libna_ref.so beside a C entry point to its calc_na_val.
if [ -f "$REF/src/na_calc.cpp" ]; then
    if "$CXX" -x c++ -std=c++17 -O2 -fPIC -w -I "$HERE/refshim/boost_include" -Dmain=na_reference_main \
           -c "$REF/src/na_calc.cpp" -o "$OUT/na_ref.o" &&
       "$CXX" -std=c++17 -O2 -fPIC -c "$HERE/refshim/ref_na_api.cpp" -o "$OUT/ref_na_api.o" &&
       "$CXX" -shared -o "$OUT/libna_ref.so" "$OUT/na_ref.o" "$OUT/ref_na_api.o"; then
        echo "build_ref: built $OUT/libna_ref.so"
    else
        echo "build_ref: na_calc not built"
    fi
fi
