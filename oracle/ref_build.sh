#!/bin/sh
# Compiles the reference channel kernels and output routines for the host,
# from their own sources where they lie, into oracle/_ref/ (TEST
# INFRASTRUCTURE ONLY).
#   ref_build.sh [REFDIR] [LX LY LZ USE_LES] ...
# The grid and the DNS/LES switch are compile-time macros of the reference
# (parameters.h); a pre-included header with the same include guard sets them.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${RR_REFERENCE_DIR:-/root/reference}/RR27V33_code_DNS_LES
OUT="$HERE/_ref"
CXX=${CXX:-g++}
if [ ! -f "$REF/collision.cu" ]; then
    echo "reference sources not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
build_one() {
    LX=$1; LY=$2; LZ=$3; LES=$4
    NAME="libref_${LX}x${LY}x${LZ}_les${LES}.so"
    P="$OUT/params_${LX}x${LY}x${LZ}_les${LES}.h"
    cat > "$P" <<EOP
#ifndef PARAMETERS_H
#define PARAMETERS_H
#define CONTINUE_STEP 50000
#define USE_LES $LES
#define LX $LX
#define LY $LY
#define LZ $LZ
#define LXYZ (LX * LY * LZ)
#define NPOP 27
#define NEND 1000000
#define NDIAG 1000
#define NFLOWOUT 100000
#define NOUT 1000
#define BLOCK_X 8
#define BLOCK_Y 8
#define BLOCK_Z 4
#endif
EOP
    # one translation unit per source file, as the reference builds them
    $CXX -O2 -fPIC -fopenmp -ffp-contract=off -std=c++14 -w -shared \
        -I "$HERE/ref_shim" -I "$REF" -include "$P" -x c++ \
        "$REF/globals.cu" "$REF/collision.cu" "$REF/streaming.cu" "$REF/macrovar.cu" \
        "$REF/BC.cu" "$REF/LES.cu" "$HERE/ref_driver.cpp" -o "$OUT/$NAME"
    echo "built $OUT/$NAME"
}
# the BGK channel program (BGK/): its kernels and its globals, one grid
build_bgk() {
    LX=$1; LY=$2; LZ=$3
    BREF=${RR_REFERENCE_DIR:-/root/reference}/BGK
    [ -f "$BREF/collision.cu" ] || return 0
    NAME="libref_bgk_${LX}x${LY}x${LZ}.so"
    P="$OUT/params_bgk_${LX}x${LY}x${LZ}.h"
    cat > "$P" <<EOP
#ifndef PARAMETERS_H
#define PARAMETERS_H
#define CONTINUE_STEP 0
#define LX $LX
#define LY $LY
#define LZ $LZ
#define LXYZ (LX * LY * LZ)
#define NPOP 27
#define NEND 10
#define NDIAG 10
#define NFLOWOUT 5000
#define NNUOUT 10
#define GRAVITY 1.0
#define BETA (0.1 / (LY * 5.0))
#define BLOCK_X 8
#define BLOCK_Y 4
#define BLOCK_Z 4
#endif
EOP
    $CXX -O2 -fPIC -fopenmp -ffp-contract=off -std=c++14 -w -shared \
        -I "$HERE/ref_shim" -I "$BREF" -include "$P" -x c++ \
        "$BREF/globals.cu" "$BREF/collision.cu" "$BREF/streaming.cu" "$BREF/macrovar.cu" \
        "$HERE/ref_driver_bgk.cpp" -o "$OUT/$NAME"
    echo "built $OUT/$NAME"
}
# the output routines (output.cu) with their globals, one grid
build_out() {
    LX=$1; LY=$2; LZ=$3; LES=$4
    NAME="libref_out_${LX}x${LY}x${LZ}_les${LES}.so"
    P="$OUT/params_${LX}x${LY}x${LZ}_les${LES}.h"
    [ -f "$P" ] || { echo "build_one $LX $LY $LZ $LES first" >&2; exit 1; }
    $CXX -O2 -fPIC -std=c++14 -w -shared \
        -I "$HERE/ref_shim" -I "$REF" -include "$P" -x c++ \
        "$REF/globals.cu" "$REF/output.cu" "$HERE/ref_output_driver.cpp" -o "$OUT/$NAME"
    echo "built $OUT/$NAME"
}
if [ $# -ge 4 ]; then
    while [ $# -ge 4 ]; do build_one "$1" "$2" "$3" "$4"; shift 4; done
else
    # grids used by the parity tests
    build_one 16 12 8 0
    build_one 16 12 8 1
    build_bgk 16 12 8
    build_out 16 12 8 1
fi
