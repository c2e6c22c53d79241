#!/bin/sh
# Builds the reference's own CPU path from its unmodified sources into
# oracle/_ref/ (git-ignored): `convert`, `main` (the reference CLIs) and
# `ref_driver` (oracle/ref_driver.cpp linked against the reference's
# graph.cpp, scd.cpp, wcc.cpp, common.cpp).  Used only to pin the oracle
# restatement, to produce tests/golden and to time the reference beside the
# restatement; it is never part of the product.  Argument 1: the reference's
# source directory (default /root/reference/src, the development container);
# where it does not exist nothing is built and the script exits 0.
# Flags: the reference's host flags without -march=native (portable) and with
# -ffp-contract=off (canonical floating-point order).
set -e
SRC=${1:-/root/reference/src}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$SRC/convert.cpp" ]; then
    echo "reference sources not found in $SRC: oracle/_ref not built"
    exit 0
fi
mkdir -p "$OUT"
up_to_date() {   # target newer than every listed source
    t=$1; shift
    [ -f "$t" ] || return 1
    for f in "$@"; do [ "$f" -nt "$t" ] && return 1; done
    return 0
}
CXX=${CXX:-g++}
FLAGS="-O3 -fopenmp -ffp-contract=off -w"
CORE="$SRC/graph.cpp $SRC/scd.cpp $SRC/wcc.cpp $SRC/common.cpp"
pids=""
up_to_date "$OUT/convert" "$SRC/convert.cpp" "$SRC/common.cpp" ||
    { $CXX $FLAGS -o "$OUT/convert" "$SRC/convert.cpp" "$SRC/common.cpp" & pids="$pids $!"; }
up_to_date "$OUT/main" "$SRC/main.cpp" $CORE ||
    { $CXX $FLAGS -o "$OUT/main" "$SRC/main.cpp" $CORE & pids="$pids $!"; }
up_to_date "$OUT/ref_driver" "$HERE/ref_driver.cpp" $CORE ||
    { $CXX $FLAGS -I"$SRC" -o "$OUT/ref_driver" "$HERE/ref_driver.cpp" $CORE & pids="$pids $!"; }
for p in $pids; do wait $p; done
echo "reference binaries in $OUT"
