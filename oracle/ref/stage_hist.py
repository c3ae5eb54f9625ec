"""Make the history-printing copy of the reference backends (test infrastructure).

The reference's tri_matrix and grid backends carry commented-out device
printfs at the point where each step's winner is known (tri_matrix.cu:235 in
reduction_blocks; grid.cu:454 before a promotion and grid.cu:462 before a
merge in reduce_recombine), and its driver enlarges the printf FIFO for them
(main.cc:28).  This script copies the staged, unmodified sources and replaces
exactly those three comment lines with a printf of the step:

    H <slot i> <slot j> <d> <px_i> <py_i> <pz_i> <E_i> <px_j> <py_j> <pz_j> <E_j>

(doubles as the hexadecimal bit patterns of their IEEE-754 encoding; i == j is
a promotion).  Nothing else changes, so the kernels take the same decisions as
the unmodified backends; the printed four-momenta let the host replay the
steps onto input labels (the slots are compacted or re-sorted by the
backends).  The output directory is git-ignored and never committed.

usage: python3 stage_hist.py <staged source dir> <output dir>
"""
import os
import shutil
import sys

HEX = "(unsigned long long)__double_as_longlong"


def _p4(expr):
    return ", ".join(f"{HEX}({expr}.{c})" for c in ("px", "py", "pz", "E"))


FMT = '"H %d %d" " %llx" " %llx %llx %llx %llx" " %llx %llx %llx %llx\\n"'

EDITS = {
    "tri_matrix.cu": [
        ('//printf("%6d%6d%6d%20.8e\\n", num_particles, i, j, min.d);',
         f"printf({FMT}, i, j, {HEX}(min.d), {_p4('jets[i]')}, {_p4('jets[j]')});"),
    ],
    "grid.cu": [
        ('//printf("will promote pseudojet %d (%d,%d) with distance %f\\n", min.j, pseudojets[min.j].u, '
         'pseudojets[min.j].v, min.distance);',
         f"printf({FMT}, min.j, min.j, {HEX}(min.distance), {_p4('pseudojets[min.j]')}, "
         f"{_p4('pseudojets[min.j]')});"),
        ('//printf("will recombine pseudojets %d (%d,%d) and %d (%d,%d) with distance %f\\n", min.i, '
         'pseudojets[min.i].u, pseudojets[min.i].v, min.j, pseudojets[min.j].u, pseudojets[min.j].v, '
         'min.distance);',
         f"printf({FMT}, min.i, min.j, {HEX}(min.distance), {_p4('pseudojets[min.i]')}, "
         f"{_p4('pseudojets[min.j]')});"),
    ],
}

COPY = ("PseudoJet.h", "cluster.h", "cudaCheck.h", "launch.h")


def main():
    src, dst = sys.argv[1], sys.argv[2]
    os.makedirs(dst, exist_ok=True)
    for f in COPY:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
    for f, edits in EDITS.items():
        with open(os.path.join(src, f)) as fh:
            lines = fh.read().split("\n")
        for old, new in edits:
            hits = [k for k, line in enumerate(lines) if line.strip() == old]
            if len(hits) != 1:
                raise SystemExit(f"stage_hist: expected one line '{old[:40]}...' in {f}, found {len(hits)}")
            k = hits[0]
            indent = lines[k][: len(lines[k]) - len(lines[k].lstrip())]
            lines[k] = indent + new
        with open(os.path.join(dst, f), "w") as fh:
            fh.write("\n".join(lines))
    print(f"staged history-printing backends into {dst}")


if __name__ == "__main__":
    main()
