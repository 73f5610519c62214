#!/bin/sh
# Builds the reference's own C kernels (algn.c with the files it #includes,
# ukkCommon.c and ukk.checkp.c behind powell_3D_align, nonaddCSc.c
# specialised to 8-, 16- and 32-bit characters by the reference's sed rule,
# avl.c and zarr.c to satisfy union.c) straight from the reference sources,
# plus oracle/ref_driver.c, into oracle/_ref/libporef.so.
# Test infrastructure only; run where the reference sources are present.
# Usage: oracle/build_ref.sh [REFERENCE_SRC_DIR]
set -e
REF="${1:-${POYD_REFERENCE_SRC:-/root/reference/src}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -f "$REF/algn.c" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
CF="-O2 -fPIC -w -I$HERE -I$REF"
LIB=libporef.so
# POYD_REF_C_PATH=1 (x86-64 only): leave __MMX__ undefined so that algn.c
# compiles its plain-C cell path (algn.c:375-453), the one an arm64 build
# uses, instead of the inline-asm one; written to libporef_cpath.so.
if [ "${POYD_REF_C_PATH:-0}" = 1 ]; then CF="$CF -mno-mmx"; LIB=libporef_cpath.so; fi
gcc -std=gnu89 -fgnu89-inline $CF -c "$REF/algn.c" -o "$OUT/algn.o"
gcc -std=gnu89 -fgnu89-inline $CF -c "$REF/avl.c" -o "$OUT/avl.o"
gcc -std=gnu89 -fgnu89-inline $CF -c "$REF/zarr.c" -o "$OUT/zarr.o"
# Powell's three-sequence alignment behind powell_3D_align
gcc -std=gnu89 -fgnu89-inline $CF -c "$REF/ukkCommon.c" -o "$OUT/ukkCommon.o"
gcc -std=gnu89 -fgnu89-inline $CF -c "$REF/ukk.checkp.c" -o "$OUT/ukkcheckp.o"
# myocamlbuild.ml.in:262-269 / 287-289: sed-specialise to CHARSIZE 8, 16 and 32
for W in 8 16 32; do
    sed -e "s/nonadd_/nonadd${W}_/g" -e "s/NONADDSIZE/${W}/g" "$REF/nonaddCSc.c" | \
        gcc -std=gnu89 -fgnu89-inline $CF -DCHARSIZE=$W -x c - -c -o "$OUT/nonadd$W.o"
done
gcc -std=gnu99 $CF -c "$HERE/ref_driver.c" -o "$OUT/ref_driver.o"
# -Bsymbolic: ukkCommon.c's step() and friends must bind to the
# reference's own definitions, not to libc's regexp step().
gcc -shared -Wl,-Bsymbolic -o "$OUT/$LIB" "$OUT/algn.o" "$OUT/avl.o" "$OUT/zarr.o" \
    "$OUT/nonadd8.o" "$OUT/nonadd16.o" "$OUT/nonadd32.o" "$OUT/ukkCommon.o" \
    "$OUT/ukkcheckp.o" "$OUT/ref_driver.o" -lm
echo "$OUT/$LIB"
