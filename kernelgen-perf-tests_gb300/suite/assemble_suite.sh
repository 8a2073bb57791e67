#!/bin/sh
# Assemble a runnable copy of the kernelgen-perf-tests suite with the b200
# (GB300) target added next to gcc and cuda.
#
#   assemble_suite.sh <reference-tree> <output-dir>
#   cd <output-dir> && ./benchmark 512 256 256 10 10 gcc b200
#
# Copies the reference tree, drops a b200/ directory (makefile + kernel file)
# into each test the target covers (the eleven stencil tests, vecadd, matvec,
# matmul, sincos, whispering), writes makefile.b200.in with this package's path, and
# applies benchmark.patch (the harness parses b200's kernel-time and regcount
# lines, as it does for cuda) and makefile.patch (%.b200 and test.b200 rules).
set -e
if [ $# -ne 2 ]; then
	echo "Usage: $0 <reference-tree> <output-dir>" >&2
	exit 1
fi
REF=$1
OUT=$2
HERE=$(cd "$(dirname "$0")" && pwd)
KG=$(cd "$HERE/.." && pwd)
if [ -e "$OUT" ]; then
	echo "$OUT exists" >&2
	exit 1
fi
cp -R "$REF" "$OUT"
chmod -R u+w "$OUT"
for t in laplacian divergence gradient uxx1 wave13pt tricubic tricubic2 jacobi lapgsrb gaussblur gameoflife \
	vecadd matvec matmul sincos whispering; do
	cp -R "$HERE/$t/b200" "$OUT/$t/b200"
done
sed "s|@KG_ROOT@|$KG|" "$HERE/makefile.b200.in" > "$OUT/makefile.b200.in"
(cd "$OUT" && patch -s -p1 < "$HERE/benchmark.patch" && patch -s -p1 < "$HERE/makefile.patch")
echo "assembled $OUT (b200 target -> $KG)"
