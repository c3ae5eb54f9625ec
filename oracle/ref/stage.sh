#!/bin/sh
# Stage the reference's unmodified CUDA/C++ sources into the git-ignored
# oracle/_ref/src so that a machine without the read-only reference mount (the
# GPU host) can compile the reference backends with oracle/ref/Makefile.
# Nothing staged here is ever committed (oracle/_ref/ is in .gitignore).
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
DST="$HERE/../_ref/src"
if [ ! -f "$REF/cluster.h" ]; then
  echo "stage.sh: no reference sources at $REF" >&2
  exit 1
fi
mkdir -p "$DST"
for f in PseudoJet.h cluster.h cudaCheck.h launch.h main.cc tri_matrix.cu n_array.cu grid.cu; do
  cp "$REF/$f" "$DST/$f"
done
echo "staged reference sources into $DST"
