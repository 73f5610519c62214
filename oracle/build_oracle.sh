#!/bin/sh
# Builds the oracle's C restatement into oracle/_build/liboracle.so.
# Test infrastructure only.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_build"
mkdir -p "$OUT"
gcc -O2 -fPIC -std=gnu99 -Wall -Wno-unused-but-set-variable -shared \
    -o "$OUT/liboracle.so" "$HERE/poy_oracle.c" -lm
echo "$OUT/liboracle.so"
