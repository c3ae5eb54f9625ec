"""Per-step phase breakdown of the shared-memory clustering kernel on the GPU.

    python -m fastjet_gpu_gb300.phases [--sizes 200,500,1000,2000,4000] [--batch 1024]

Builds the phase-counter variant of the library (-DFJG_PHASE_CLOCKS, into
fastjet_gpu_gb300/_lib_phases/; the product build is untouched) and loads it
in place of the product library.  It then clusters lone events of the given
sizes, one event per launch (anti-kt R=0.4; the plain path, where a step's
latency is the event's critical path), and one batch of mixed events of
50-2000 particles (several CTAs per SM, the throughput path).  For each it
prints the clock cycles per merge step of each phase, as counted by the
kernel's clock64() phase counters:

  s1_argmin      argmin of the keys, up to its decision (barrier B1)
  s2_merge       the merge: new jet's kinematics || target scans, up to B2
  s3_new_jet     every slot against the new jet, targets finished, up to B3
  tail_resolve   the new jet's neighbour, up to the next step
  kin_warp0..2   inside s2_merge: each merge warp's kinematics chain
                 (azimuth; rapidity and momentum; weight and history)
  rescan_s2      inside s2_merge: the first rescan thread's work
"""
from __future__ import annotations

import argparse
import json
import sys


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="200,500,1000,2000,4000")
    ap.add_argument("--batch", type=int, default=1024, help="events of the mixed batch (0: none)")
    ap.add_argument("--algo", type=int, default=-1)
    ap.add_argument("--radius", type=float, default=0.4)
    args = ap.parse_args()

    from fastjet_gpu_gb300 import build as B
    lib = B.build(phase_clocks=True)
    import fastjet_gpu_gb300 as F
    F.LIB_PATH = lib
    import torch

    from fastjet_gpu_gb300 import events as E

    ctx = F.Context(0)
    names = [k for k in F.Context.PHASES if k not in ("steps", "events")]
    rows = []

    def report(tag, c):
        steps = max(c["steps"], 1)
        row = {"case": tag, "steps": c["steps"], "events": c["events"]}
        row.update({k: c[k] / steps for k in names})
        row["step_total"] = sum(row[k] for k in ("s1_argmin", "s2_merge", "s3_new_jet", "tail_resolve"))
        rows.append(row)
        print(f"{tag:>28}: " + "  ".join(f"{k} {row[k]:8.0f}" for k in names + ["step_total"]), flush=True)

    for n in [int(x) for x in args.sizes.split(",") if x]:
        ev = torch.from_numpy(E.single_event(n, 3, seed=900 + n)).cuda()
        ctx.cluster_event(ev, args.algo, args.radius)
        ctx.phase_clocks(reset=True)
        for _ in range(3):
            ctx.cluster_event(ev, args.algo, args.radius)
        report(f"lone event, {n} particles", ctx.phase_clocks(reset=True))
    if args.batch:
        b = E.mixed_batch(args.batch, 50, 2000, seed=3)
        p4 = torch.from_numpy(b.particles).cuda()
        off = torch.from_numpy(b.offsets).cuda()
        ctx.cluster_batch_device(p4, off, args.algo, args.radius)
        torch.cuda.synchronize()
        ctx.phase_clocks(reset=True)
        ctx.cluster_batch_device(p4, off, args.algo, args.radius)
        torch.cuda.synchronize()
        report(f"batch of {args.batch}, 50-2000", ctx.phase_clocks(reset=True))
    ctx.close()
    print(json.dumps({"phase_cycles_per_step": rows, "algo": args.algo, "R": args.radius,
                      "gpu": torch.cuda.get_device_name(0)}))


if __name__ == "__main__":
    sys.exit(main())
