"""Many boxes of uneven HII_DIM in one persistent launch (no counterpart in the reference, whose
``find_HII_bubbles.py`` runs one box per call).

``python -m 21cmpy_gb300.Programs.batch_sweep [--boxes K] [--schedule LxC | --tune] [--runs R]
[--products] [--profile]`` builds the first K boxes of the uneven parameter sweep (HII_DIM ~
U{64, 96, 128, 160}, BOX_LEN = 1.5 HII_DIM Mpc, zeta ~ U[10, 80], R_mfp ~ U[5, 50] Mpc,
log10 T_vir ~ U[4, 5.3], z ~ U[6, 10]), runs them R times through ``BatchedExcursionSet``
(graph replays) and prints one JSON line: milliseconds per batch, voxel-radius updates per
second, the work-queue schedule and, with ``--profile``, the share of CTA time and the clock
cycles per tile of every pass kind.  ``--products`` adds delta_T and the 20-bin P(k) of every box
to the launch.
"""
from __future__ import annotations

import argparse
import json


def main(argv=None):
    import torch

    from .. import autotune, batch, cosmology, grf, schedule
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--boxes", type=int, default=64)
    ap.add_argument("--schedule", default=None, help="LANESxTILES_PER_TICKET, e.g. 0x16 (default: the library's)")
    ap.add_argument("--tune", action="store_true", help="time the autotuner's schedules first and keep the best")
    ap.add_argument("--runs", type=int, default=5)
    ap.add_argument("--products", action="store_true", help="also delta_T and P(k) of every box")
    ap.add_argument("--profile", action="store_true", help="per-pass cycle counters (one extra launch)")
    args = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    specs = grf.uneven_batch()[:args.boxes]
    boxes = batch.boxes_from_specs(specs, dev)
    kw = {}
    if args.products:
        kw["t_factors"] = [cosmology.brightness_temperature_factor(st.z, cosmology.BASELINE_COSMO) for _, st in boxes]
        kw["pk_edges"] = [schedule.pk_edges(st.n, st.box_len, 20) for _, st in boxes]
    with batch.BatchedExcursionSet(boxes, use_graph=True, device=dev, **kw) as b:
        if args.schedule:
            lanes, chunk = (int(v) for v in args.schedule.lower().split("x"))
            b.set_schedule(lanes, chunk)
        tuned = autotune.tune_batch(b) if args.tune else None
        b.run()
        b.check()
        stream = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.runs):
            b.run()
        e1.record(stream)
        e1.synchronize()
        b.check()
        ms = e0.elapsed_time(e1) / args.runs
        out = {"boxes": len(boxes), "ms_per_batch": ms,
               "voxel_radius_updates_per_s": b.voxel_radius_updates() / (ms * 1e-3), **b.info()}
        if tuned:
            out["tuned_ms"] = {f"{k[0]}x{k[1]}": round(v, 3) for k, v in tuned.items()}
        if args.profile:
            b.profile(True)
            b.run()
            prof = b.profile_read()
            b.profile(False)
            total = sum(v["tile_cycles"] + v["wait_cycles"] for v in prof.values())
            out["profile"] = {k: {"share": round((v["tile_cycles"] + v["wait_cycles"]) / total, 4),
                                  "wait_share": round(v["wait_cycles"] / total, 4),
                                  "tiles": v["tiles"], "cycles_per_tile": round(v["tile_cycles"] / v["tiles"])}
                              for k, v in prof.items()}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
