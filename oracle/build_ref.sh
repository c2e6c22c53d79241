#!/bin/sh
# Builds the reference's own CPU path from its unmodified sources into
# oracle/_ref/ (git-ignored): `convert`, `main` (the reference CLIs) and
# `ref_driver` (oracle/ref_driver.cpp linked against the reference's
# graph.cpp, scd.cpp, wcc.cpp, common.cpp).  Used only to pin the oracle
# restatement and to produce tests/golden; needs the reference sources
# (argument 1, default /root/reference/src), so it runs in the development
# container only.  Flags: the reference's host flags without -march=native
# (portable) and with -ffp-contract=off (canonical floating-point order).
set -e
SRC=${1:-/root/reference/src}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O3 -fopenmp -ffp-contract=off -w"
$CXX $FLAGS -o "$OUT/convert" "$SRC/convert.cpp" "$SRC/common.cpp" & p1=$!
$CXX $FLAGS -o "$OUT/main" "$SRC/main.cpp" "$SRC/graph.cpp" "$SRC/scd.cpp" "$SRC/wcc.cpp" "$SRC/common.cpp" & p2=$!
$CXX $FLAGS -I"$SRC" -o "$OUT/ref_driver" "$HERE/ref_driver.cpp" "$SRC/graph.cpp" "$SRC/scd.cpp" "$SRC/wcc.cpp" "$SRC/common.cpp" & p3=$!
wait $p1
wait $p2
wait $p3
echo "reference binaries in $OUT"
