"""Per-step phase breakdown of the shared-memory clustering kernel on the GPU.

    python -m fastjet_gpu_gb300.phases [--sizes 200,500,1000,2000,4000] [--batch 1024]

Builds the phase-counter variant of the library (-DFJG_PHASE_CLOCKS, into
fastjet_gpu_gb300/_lib_phases/; the product build is untouched) and loads it
in place of the product library.  It then clusters lone events of the given
sizes, one event per launch (anti-kt R=0.4; the plain path, where a step's
latency is the event's critical path; above 4096 particles pile-up-like
events on the tiled kernel), and one batch of mixed events of 50-2000
particles (several CTAs per SM, the throughput path).  For each it prints the
clock cycles per merge step of each phase, as counted by the kernels'
clock64() phase counters.  Shared-memory kernel:

  s1_argmin      argmin of the keys, up to its decision (barrier B1)
  s2_merge       the merge: new jet's kinematics || target scans, up to B2
  s3_new_jet     every slot against the new jet, targets finished, up to B3
  tail_resolve   the new jet's neighbour, up to the next step
  kin_warp0..2   inside s2_merge: each merge warp's kinematics chain
                 (azimuth; rapidity and momentum; weight and history)
  rescan_s2      inside s2_merge: the first rescan thread's work
  exact_*        FP64 fallbacks per step: argmin not certified, a slot's
                 closer-than-its-neighbour test, a key's pair-or-beam choice,
                 a neighbour search whose certificate failed

Tiled kernel: t_rebuild (tile-list rebuilds, per step), t_s1_argmin (over the
tile summaries), t_s2_merge_detect (merge || target detection and scans),
t_s3_lists_targets_window (list update, targets, the new jet against its
window), t_s3_overflow (targets beyond the listed ones, flags), t_s3c_summaries (changed tiles, the new jet's neighbour); inside t_s2:
t_kin_rapidity (the rapidity chain) and t_detect_s2 (the first detection
thread's work); inside t_s3: t_list_update (thread 0), t_targets_warp1 (warp
1's targets), t_window_thread0 (thread 0's share of the window pass); inside
t_s3c_summaries: t_resolve_new_jet and t_summary_new_jet_tile (warp 0: its
wait for warp 1 and the merge of the new jet's key), t_summaries_warp1 (warp 1:
the new jet's tile without the new jet, or on promotion steps its share of the
changed tiles).
"""
from __future__ import annotations

import argparse
import json
import sys


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="200,500,1000,2000,4000,10000,40000")
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
    small = ["s1_argmin", "s2_merge", "s3_new_jet", "tail_resolve", "kin_warp0", "kin_warp1", "kin_warp2",
             "rescan_s2"]
    tiled = ["t_rebuild", "t_s1_argmin", "t_s2_merge_detect", "t_s3_lists_targets_window", "t_s3_overflow",
             "t_s3c_summaries", "t_kin_rapidity", "t_detect_s2", "t_list_update", "t_targets_warp1",
             "t_window_thread0", "t_resolve_new_jet", "t_summary_new_jet_tile", "t_summaries_warp1"]
    rows = []

    def report(tag, c):
        row = {"case": tag}
        if c["steps"]:
            steps = c["steps"]
            row.update({"steps": steps, "events": c["events"]})
            row.update({k: c[k] / steps for k in small})
            row["step_total"] = sum(row[k] for k in ("s1_argmin", "s2_merge", "s3_new_jet", "tail_resolve"))
            # FP64 fallbacks per step (the FP32 intervals could not decide)
            row.update({k: c[k] / steps for k in ("exact_argmin", "exact_closer", "exact_key", "exact_nn")})
            print(f"{tag:>28}: " + "  ".join(f"{k} {row[k]:8.0f}" for k in small + ["step_total"]) +
                  "  per step: " + "  ".join(f"{k} {row[k]:.3f}" for k in
                                            ("exact_argmin", "exact_closer", "exact_key", "exact_nn")), flush=True)
        if c["t_steps"]:
            steps = c["t_steps"]
            row.update({"t_steps": steps, "t_events": c["t_events"]})
            row.update({k: c[k] / steps for k in tiled})
            row["t_step_total"] = sum(row[k] for k in tiled[:6])
            row["t_targets_per_step"] = c["t_targets"] / steps
            row["t_steps_with_targets"] = c["t_target_steps"] / steps
            print(f"{tag:>28}: " + "  ".join(f"{k} {row[k]:8.0f}" for k in tiled + ["t_step_total"]) +
                  f"  targets per step {row['t_targets_per_step']:.2f}, steps with targets "
                  f"{row['t_steps_with_targets']:.2f}", flush=True)
        rows.append(row)

    for n in [int(x) for x in args.sizes.split(",") if x]:
        gen = E.single_event(n, 3, seed=900 + n) if n <= 4096 else E.portable_event(n, 4, seed=900 + n)
        ev = torch.from_numpy(gen).cuda()
        ctx.cluster_event(ev, args.algo, args.radius)
        ctx.phase_clocks(reset=True)
        for _ in range(3 if n <= 4096 else 1):
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
