#!/bin/sh
# Stage the reference's unmodified CUDA/C++ sources into the git-ignored
# oracle/_ref/src so that a machine without the reference sources (the GPU
# host) can compile the reference backends with oracle/ref/Makefile, and make
# the history-printing copy in oracle/_ref/hist_src (stage_hist.py).
# Nothing staged here is ever committed (oracle/_ref/ is in .gitignore).
#
# usage: sh oracle/ref/stage.sh <reference source directory>
set -e
REF=${1:?usage: stage.sh <reference source directory>}
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
python3 "$HERE/stage_hist.py" "$DST" "$HERE/../_ref/hist_src"
