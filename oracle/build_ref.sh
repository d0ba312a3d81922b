#!/bin/sh
# Builds the reference's own code from its sources into oracle/_ref/ (git-ignored).  Test
# infrastructure only: the outputs are oracles, never part of the product.
#
#   fromDirectToUndirect, preprocess        Preprocess/compile.sh:1-2 (text edge list -> CSR)
#   TransformTxt2Binary, preprocess_out     Preprocess/speedupIO/preprocess.sh:2-3 (large graphs)
#   partition                               Preprocess/partition.cpp; mapvertex (:131-165) falls
#                                           off the end of an int function, which GCC 13 turns
#                                           into a trap, so a patched copy is compiled from a
#                                           temporary directory outside the repository
#   tc_ref_w.cubin                          Without-graph-partition/TC.cu device code for
#                                           sm_103a; loaded on the GPU host by ref_tc_driver.c
#                                           (the x86 host binaries here do not run there)
#
# Usage: oracle/build_ref.sh [<reference_root>]
# Without an argument the reference is looked for at /root/reference, where the build container
# mounts it; where it is absent (the GPU host, which uses the files built here) nothing is built.
set -eu
[ $# -le 1 ] || { echo "usage: $0 [<reference_root>]" >&2; exit 2; }
if [ $# -eq 1 ]; then
  REF=$1
else
  REF=/root/reference
  [ -d "$REF/Preprocess" ] || exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -d "$REF/Preprocess" ] || { echo "reference sources not found at $REF" >&2; exit 1; }

g++ -O3 -w "$REF/Preprocess/fromDirectToUndirect.cpp" -o "$OUT/fromDirectToUndirect"
g++ -O3 -w "$REF/Preprocess/preprocess_outdegree.cpp" -o "$OUT/preprocess"
g++ -O3 -w "$REF/Preprocess/speedupIO/TransformTxt2Binary.cpp" -o "$OUT/TransformTxt2Binary"
g++ -O3 -w "$REF/Preprocess/speedupIO/preprocess_out.cpp" -o "$OUT/preprocess_out"

TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
sed '165s/^}/    return 0;\n}/' "$REF/Preprocess/partition.cpp" > "$TMP/partition.cpp"
grep -q 'return 0;' "$TMP/partition.cpp"
g++ -O3 -w "$TMP/partition.cpp" -o "$OUT/partition"

if command -v nvcc >/dev/null 2>&1; then
  nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w \
    -I"$REF/Without-graph-partition" "$REF/Without-graph-partition/TC.cu" -o "$OUT/tc_ref_w.cubin"
fi
echo "reference oracles built in $OUT"
