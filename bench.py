#!/usr/bin/env python
"""Excursion-set benchmark: voxel-radius updates/s of the HII_DIM=256 sweep on GB300.

Workload (one step): 52 density boxes of 256^3 cells, BOX_LEN = 300 Mpc (seeds 0-3 x z = 6.0,
6.5, ..., 12.0, Gaussian random fields with the BBKS spectrum), each run through the whole path:
forward transform, 32 radii of the excursion-set loop (zeta = 30, R_mfp = 15 Mpc,
Tvir = 1e4 K, real-space top-hat), final partial ionisation, delta_T and a 20-bin P(k).

Printed JSON line (rank 0): ``value`` = voxel-radius updates / s with inputs resident in HBM,
``e2e`` = the same metric through ``Programs.pipeline.simulate_box`` with pinned host buffers
(host<->device copies inside the timed region), ``roofline`` for the dominant kernel from
per-launch CUDA events over the timed region, ``cpu_baseline`` = the FP64 numpy oracle on a
bounded sample of the same workload on the host cores.

``--impl reference`` times the oracle port of the reference path (there is no runnable
reference implementation: Python 2 + PyCUDA + pyfft + cosmolopy) on all host cores instead.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-radius updates/s @256^3 (fused excursion-set engine)"
UNIT = "voxel-radius updates/s"
N = 256
BOX_LEN = 300.0
LANES = 3                 # boxes in flight per GPU, each on its own plan and stream
NUM_BINS = 20

# Algorithmic bytes per voxel for one launch of each kernel kind: what the kernel must read and
# write at minimum (half spectrum = 8 B x (N/2+1)/N per real voxel, ~4.03 B at 256^3).
HALF = 8.0 * (N // 2 + 1) / N


def kernel_bytes_per_voxel() -> dict:
    return {
        "col_z_inv_filter": 2 * HALF,                 # read spectrum, write filtered intermediate
        "col_y_inv": 2 * HALF,                        # read + write intermediate
        # read spectrum, write delta_R, read previous delta_R; in centre mode the flags travel in
        # delta_R's lowest mantissa bit, so no bitmap is read or written
        "row_c2r_ionize": HALF + 4 + 4,
        "row_r2c": 4 + HALF,
        "col_y_fwd": 2 * HALF,
        "col_z_fwd": 2 * HALF,
        "final": 4 + 4,                               # read final delta_R (flags in it), write x_HI
        "delta_T": 12.0,
        "row_r2c_pk": 4 + HALF,
        "col_z_fwd_pk": HALF,
        "filter_table": 0.0,
    }


# whole-path algorithmic bytes: 22 B per voxel-radius, 20 B per voxel-box (forward transform +
# x_HI write), 24 B per voxel for delta_T and P(k)
B_RADIUS, B_BOX, B_DT_PK = 22.0, 20.0, 24.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i - 5] for r in self.rows for i in range(5, 9) if r[i].lower() == "active"})
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_workload(rank: int, world: int, boxes: int):
    """This rank's boxes: the sweep widened to 4 seeds per GPU, split over ranks by cost N^3 * N_R
    (batch.shard_specs); with every box of equal cost each rank gets one full 52-box sweep."""
    grf = importlib.import_module("21cmpy_gb300.grf")
    batch = importlib.import_module("21cmpy_gb300.batch")
    specs = grf.sweep_256(seeds=range(4 * world))
    mine = [specs[i] for i in batch.shard_specs(specs, world)[rank]][:boxes]
    base = {}
    out = []
    for s in mine:
        if s.seed not in base:
            base[s.seed] = grf.grf_z0(s.n, s.box_len, s.seed)
        out.append((s, s.seed, grf.density_box(s.n, s.box_len, s.seed, s.z, base=base[s.seed])))
    return out


def sweep_config(nboxes: int, radii_per_box: int, world: int) -> dict:
    """The workload both arms report (the reference arm times a bounded sample of it)."""
    return {"workload": f"excursion-set sweep: {nboxes} boxes of 256^3 per GPU (seeds 0-3 x z=6.0..12.0 step 0.5), "
                        "BOX_LEN=300 Mpc, zeta=30, R_mfp=15 Mpc, Tvir=1e4 K, real-space top-hat, "
                        f"{radii_per_box} radii/box, delta_T + {NUM_BINS}-bin P(k)",
            "n": N, "box_len_mpc": BOX_LEN, "boxes_per_gpu": nboxes, "radii_per_box": radii_per_box,
            "l2": "no flush: every box's inputs (64 MiB density + 64 MiB spectrum) and its 256 MiB working "
                  "set exceed the 129 MB L2, and consecutive boxes touch different inputs",
            "parallelism": f"{world} independent GPU(s), 4 seeds x 13 redshifts per GPU split by cost N^3 N_R "
                           f"(batch.shard_specs), no collective; {LANES} boxes side by side per GPU "
                           "(one plan and stream each)"}


def setups_for(work):
    cos = importlib.import_module("21cmpy_gb300.cosmology")
    sch = importlib.import_module("21cmpy_gb300.schedule")
    res = []
    for s, _seed, _d in work:
        st = sch.ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min, R_max=s.R_max,
                              cosmo=cos.BASELINE_COSMO)
        res.append((st, cos.brightness_temperature_factor(s.z, cos.BASELINE_COSMO)))
    return res


def oracle_box(O, d, st, c, edges, backend="numpy", workers=1):
    """One box of the sweep on the host: every radius, the final step, delta_T and P(k)."""
    ion = O.conv_bubbles(d, st, backend=backend, workers=workers)["ionized"]
    dT, ave = O.delta_T(1.0 - ion, d, c)
    O.power_spectrum(dT, ave, BOX_LEN, edges, backend=backend, workers=workers)


def cpu_baseline(work, setups) -> dict:
    """FP64 numpy oracle (numpy.fft, one thread) on one whole box of the sweep."""
    from oracle import es_oracle as O
    sch = importlib.import_module("21cmpy_gb300.schedule")
    s, seed, d = work[0]
    st, c = setups[0]
    edges = sch.pk_edges(N, BOX_LEN, NUM_BINS)
    t0 = time.perf_counter()
    oracle_box(O, d, st, c, edges)
    dt = time.perf_counter() - t0
    return {"value": N ** 3 * st.n_radii / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"one whole 256^3 box of the sweep (seed {seed}, z={s.z}): forward FFT, all {st.n_radii} "
                      f"radii, final step, delta_T and {NUM_BINS}-bin P(k); numpy.fft float64, one thread, {dt:.1f} s"}


def run_reference(args):
    """Reference arm: the oracle port of the path on all host cores (scipy.fft workers and a thread
    pool over slabs for the per-radius elementwise work), one whole box of the sweep per step."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from oracle import es_oracle as O
    sch = importlib.import_module("21cmpy_gb300.schedule")
    # a few distinct boxes of rank 0's sweep, taken in turn (every box has the same radius count)
    distinct = max(1, min(4, args.warmup + args.steps))
    work = make_workload(0, world, distinct)
    setups = setups_for(work)
    edges = sch.pk_edges(N, BOX_LEN, NUM_BINS)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    # the config of the GPU arm at the same world size: the full sweep's box and radius counts
    grf = importlib.import_module("21cmpy_gb300.grf")
    full = grf.sweep_256()[:args.boxes]
    radii = setups[0][0].n_radii
    config = sweep_config(len(full), radii, world)
    count = [0]

    def step():
        i = count[0] % len(work)
        count[0] += 1
        st, c = setups[i]
        oracle_box(O, work[i][2], st, c, edges, backend="scipy", workers=cores)
        return st.n_radii

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    updates = 0
    for _ in range(args.steps):
        updates += N ** 3 * step()
    dt = time.perf_counter() - t0
    value = updates / dt
    sample = (f"one whole box of the {len(full)}-box sweep per step ({len(work)} distinct boxes taken in turn): "
              f"forward FFT, all {radii} of {radii} radii, final step, delta_T and {NUM_BINS}-bin P(k); float64, "
              f"scipy.fft and the per-radius window / erfc / threshold slabs on {cores} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded BBKS Gaussian random fields, Om=0.31 Ob=0.049 h=0.68 s8=0.81)",
            "config": config,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--boxes", type=int, default=52, help="boxes per step (the sweep has 52)")
    ap.add_argument("--plan-config", default=None,
                    help="apply this plan configuration (8 comma-separated integers, the autotuner's "
                         "tuple) instead of tuning: makes a profiled run's launch sequence fixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the uneven batched-sweep measurement")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate-speed measurement")
    ap.add_argument("--no-perturb", action="store_true", help="skip the density-evolution measurement")
    ap.add_argument("--no-config3", action="store_true", help="skip the single 512^3 box measurement")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(dev)

    import __graft_entry__
    __graft_entry__.build()
    eng = importlib.import_module("21cmpy_gb300.engine")
    sch = importlib.import_module("21cmpy_gb300.schedule")

    work = make_workload(rank, world, args.boxes)
    setups = setups_for(work)
    edges = sch.pk_edges(N, BOX_LEN, NUM_BINS)
    nboxes = len(work)
    dens = [torch.from_numpy(d).to(dev) for _s, _seed, d in work]
    xh = [torch.empty((N, N, N), dtype=torch.float32, device=dev) for _ in range(nboxes)]
    dT = [torch.empty((N, N, N), dtype=torch.float32, device=dev) for _ in range(nboxes)]
    nf = torch.empty((nboxes, 1), dtype=torch.float32, device=dev)
    ave = torch.empty((nboxes, 1), dtype=torch.float32, device=dev)
    pk = torch.empty((nboxes, 3, NUM_BINS), dtype=torch.float32, device=dev)
    at = importlib.import_module("21cmpy_gb300.autotune")
    plan = eng.ExcursionSetPlan(N, BOX_LEN, max_radii=64, device=dev)
    if args.plan_config:
        cfg = tuple(int(v) for v in args.plan_config.split(","))
        if len(cfg) != 8:
            ap.error("--plan-config needs 8 integers")
        at.apply(plan, cfg)
        tuned = {"config": list(cfg), "source": "given"}
    else:
        tuned = at.ensure_tuned(plan)
    # boxes are independent: LANES plans, each on its own stream, take boxes in turn
    plans = [plan] + [eng.ExcursionSetPlan(N, BOX_LEN, max_radii=64, device=dev) for _ in range(LANES - 1)]
    for p_ in plans[1:]:
        at.apply(p_, tuned["config"])
    lane_streams = [torch.cuda.Stream(dev) for _ in plans]
    updates_per_step = sum(N ** 3 * st.n_radii for st, _c in setups)

    def step():
        main = torch.cuda.current_stream(dev)
        fork = torch.cuda.Event()
        fork.record(main)
        for s_ in lane_streams:
            s_.wait_event(fork)
        for i in range(nboxes):
            st, c = setups[i]
            p_, s_ = plans[i % LANES], lane_streams[i % LANES]
            p_.run(dens[i], st, out=xh[i], nf=nf[i], stream=s_)
            p_.delta_T(xh[i], dens[i], c, out=dT[i], ave=ave[i], stream=s_)
            p_.power_spectrum(dT[i], ave[i], edges, out=pk[i], stream=s_)
        for s_ in lane_streams:
            main.wait_stream(s_)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        step()
    barrier()
    stream = torch.cuda.current_stream(dev)
    clocks = ClockSampler(dev.index)
    clocks.start()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # timed region: the whole sweep, K steps, no per-launch instrumentation
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    # the same K steps again with a CUDA event pair around every launch on the plan's stream: the
    # per-kernel times (kernel_ms, roofline) of this instrumented pass
    launches_per_box = 3 + 1 + 3 * max(st.n_radii for st, _c in setups) + 1 + 1 + 3
    for p_ in plans:
        p_.profile_enable(launches_per_box * nboxes * args.steps + 16)
    barrier()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.steps):
        step()
    e3.record(stream)
    barrier()
    elapsed_profiled = e2.elapsed_time(e3) / 1e3
    clock_info = clocks.stop()
    prof = {}
    for p_ in plans:
        for k, (ms_, cnt_) in p_.profile_read().items():
            a_ms, a_cnt = prof.get(k, (0.0, 0))
            prof[k] = (a_ms + ms_, a_cnt + cnt_)
        p_.profile_enable(0)
    if dist is not None:
        t = torch.tensor([elapsed], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = updates_per_step * world * args.steps / elapsed

    # dominant kernel roofline from the per-launch events of the timed region
    hbm, peak_kind = peaks()
    bpv = kernel_bytes_per_voxel()
    dom = max((k for k in prof if k in bpv), key=lambda k: prof[k][0])
    dom_ms, dom_count = prof[dom]
    dom_bytes = bpv[dom] * N ** 3
    achieved = dom_bytes * dom_count / (dom_ms / 1e3) / 1e9
    traffic = measured_traffic(dom)
    radii_total = sum(st.n_radii for st, _c in setups)
    path_bytes = (B_RADIUS * N ** 3 * radii_total + (B_BOX + B_DT_PK) * N ** 3 * nboxes) * args.steps * world
    path_gbs = path_bytes / elapsed / 1e9

    # boxes run side by side and, with overlapped radii, the row pass shares the GPU with the next
    # radius' column passes, so live launch times include co-running work; one more instrumented
    # step, boxes in turn on one plan with the overlap off, gives the same kernel's time alone
    lib_consts = importlib.import_module("21cmpy_gb300._lib")
    overlapped = plan.get_option(lib_consts.OPT_OVERLAP) == 1 or LANES > 1
    roofline_isolated = None
    if overlapped:
        ov_old = plan.get_option(lib_consts.OPT_OVERLAP)
        plan.set_option(lib_consts.OPT_OVERLAP, 0)
        plan.profile_enable(launches_per_box * nboxes + 16)
        barrier()
        for i in range(nboxes):
            st, c = setups[i]
            plan.run(dens[i], st, out=xh[i], nf=nf[i])
            plan.delta_T(xh[i], dens[i], c, out=dT[i], ave=ave[i])
            plan.power_spectrum(dT[i], ave[i], edges, out=pk[i])
        barrier()
        prof_iso = plan.profile_read()
        plan.profile_enable(0)
        plan.set_option(lib_consts.OPT_OVERLAP, ov_old)
        iso_ms, iso_count = prof_iso[dom]
        iso_gbs = dom_bytes * iso_count / (iso_ms / 1e3) / 1e9
        roofline_isolated = {"kernel": dom, "achieved": iso_gbs, "peak": hbm, "unit": "GB/s", "frac": iso_gbs / hbm,
                             "launch_ms": iso_ms / iso_count}

    # end-to-end through the public host-buffer API (pinned host inputs/outputs)
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, work, dev, barrier, dist)

    batch_info = None
    if not args.no_batch and world == 1:
        batch_info = run_batch(args, dev)

    surrogate_info = None
    if not args.no_surrogate and world == 1:
        surrogate_info = run_surrogate(dev)
    config3_info = None
    if not args.no_config3 and world == 1:
        config3_info = run_config3(dev, hbm)
    perturb_info = None
    if not args.no_perturb and world == 1:
        perturb_info = run_perturb(dev, hbm)
        perturb_info["initial_conditions"] = run_initial(dev)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded BBKS Gaussian random fields, Om=0.31 Ob=0.049 h=0.68 s8=0.81)",
        "config": sweep_config(nboxes, radii_total // nboxes, world),
        "gpu_launches": int(sum(c for _ms, c in prof.values())),
        "autotune": {"config": tuned.get("config"), "source": tuned.get("source"),
                     "meaning": "(pass variant, column tile, row tile, column radix schedule, row radix schedule, overlapped radii, row-pass CTAs per SM, column-pass CTAs per SM)"},
        "kernel_ms": {k: round(v[0], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "kernel_ms_note": f"per-launch CUDA events over a second pass of the same {args.steps} steps "
                          f"({1e3 * elapsed_profiled / args.steps:.1f} ms per step with the events)"
                          + (f"; {LANES} boxes run side by side on their own plans and streams, and radii overlap "
                             "(column passes of radius r + 1 beside the row pass of radius r), so a launch's time "
                             "includes the work running beside it" if overlapped else ""),
        "roofline": roofline_line(dom, dom_bytes, dom_ms, dom_count, achieved, hbm, peak_kind, traffic,
                                  roofline_isolated, prof, elapsed_profiled, args.steps),
        "path_roofline": {"achieved": path_gbs, "peak": hbm, "unit": "GB/s", "frac": path_gbs / hbm,
                          "bytes_model": "22 B/voxel-radius + 20 B/voxel-box + 24 B/voxel delta_T+P(k)"},
        "clocks": clock_info,
    }
    if e2e is not None:
        line["e2e"] = e2e
    if batch_info is not None:
        line["batched_sweep"] = batch_info
    if surrogate_info is not None:
        line["surrogate"] = surrogate_info
    if config3_info is not None:
        line["box_512"] = config3_info
    if perturb_info is not None:
        line["perturb_field"] = perturb_info
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(work, setups)
    if rank == 0:
        print(json.dumps(line), flush=True)
    for p_ in plans:
        p_.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0



def roofline_line(dom, dom_bytes, dom_ms, dom_count, achieved, hbm, peak_kind, traffic, iso, prof,
                  elapsed_profiled, steps):
    """The dominant kernel's roofline.  With boxes side by side and overlapped radii, an event pair
    around a launch also spans the work of the other streams, so the kernel's own rate comes from
    one extra step run serially (one plan, boxes in turn, radii not overlapped); the live
    event-bracketed rate and the wall time apportioned by the kernel's share of event time are
    given beside it."""
    live = {"achieved": achieved, "frac": achieved / hbm, "launch_ms": dom_ms / dom_count,
            "measured": "CUDA event pair around each launch in the instrumented pass of the concurrent "
                        "schedule (spans the work running beside it on other streams)"}
    share = dom_ms / sum(ms for ms, _c in prof.values())
    app_ms = 1e3 * elapsed_profiled * share / dom_count
    apportioned = {"achieved": dom_bytes / (app_ms / 1e3) / 1e9, "frac": dom_bytes / (app_ms / 1e3) / 1e9 / hbm,
                   "launch_ms": app_ms, "share_of_event_time": share,
                   "measured": "wall time of the instrumented pass times the kernel's share of all launches' "
                               "event time, per launch"}
    line = {"bound": "hbm", "kernel": dom, "peak": hbm, "unit": "GB/s", "peak_source": f"{peak_kind} hbm_gbs",
            "algorithmic_bytes_per_launch": dom_bytes, "traffic": traffic}
    if iso is None:
        line.update({"achieved": achieved, "frac": achieved / hbm, "launch_ms": dom_ms / dom_count,
                     "measured": "CUDA event pair around each launch, instrumented pass of the same steps"})
        return line
    line.update({"achieved": iso["achieved"], "frac": iso["frac"], "launch_ms": iso["launch_ms"],
                 "measured": "CUDA event pair around each launch of one extra step of the same boxes run "
                             "serially on one plan (boxes in turn, radii not overlapped): the kernel alone",
                 "live": live, "apportioned": apportioned})
    return line

def run_e2e(args, work, dev, barrier, dist):
    import torch
    pipe = importlib.import_module("21cmpy_gb300.Programs.pipeline")
    cos = importlib.import_module("21cmpy_gb300.cosmology")
    params = {"ZETA": 30.0, "ION_Tvir_MIN": 1e4, "R_BUBBLE_MAX": 15.0, "R_BUBBLE_MIN": 0.5, "DELTA_R_FACTOR": 1.1,
              "COSMO": cos.BASELINE_COSMO, "NUM_BINS": NUM_BINS, "DIMENSIONAL_T_POWER_SPEC": False}
    host_in = [torch.from_numpy(d).pin_memory() for _s, _seed, d in work]
    xh_out = [torch.empty((N, N, N), dtype=torch.float32).pin_memory() for _ in work]
    dT_out = [torch.empty((N, N, N), dtype=torch.float32).pin_memory() for _ in work]
    pd = {"BoxSize": BOX_LEN, "HIIdim": N}

    zs = [s.z for s, _seed, _d in work]

    def step():
        res = pipe.simulate_sweep(host_in, pd, zs, fil=0, params=params, xH_outs=xh_out, dT_outs=dT_out, device=dev)
        return sum(r["n_radii"] for r in res)

    for _ in range(3):
        step()
    barrier()
    t0 = time.perf_counter()
    radii = 0
    for _ in range(args.steps):
        radii += step()
    barrier()
    dt = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([dt], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
    world = dist.get_world_size() if dist is not None else 1
    nb = len(work)
    return {"value": N ** 3 * radii * world / dt, "unit": UNIT, "h2d_bytes_per_step": nb * N ** 3 * 4,
            "d2h_bytes_per_step": nb * (2 * N ** 3 * 4 + 3 * NUM_BINS * 4 + 8),
            "api": "Programs.pipeline.simulate_sweep (find_HII_bubbles + delta_T of every box on pinned host "
                   "buffers, copies overlapped with compute, 3 boxes side by side)",
            "ms_per_step": 1e3 * dt / args.steps}



def run_config3(dev, hbm_gbs: float, reps: int = 3):
    """One 512^3 box (BOX_LEN = 600 Mpc, z = 7.5, zeta = 40, R_mfp = 30 Mpc, 40 radii): time per box,
    per-pass HBM GB/s from one serial instrumented box, and the engine's plain 3-D real FFTs next to
    torch.fft (cuFFT), which is timed here as a yardstick only."""
    import numpy as np
    import torch
    eng = importlib.import_module("21cmpy_gb300.engine")
    at = importlib.import_module("21cmpy_gb300.autotune")
    grf = importlib.import_module("21cmpy_gb300.grf")
    sch = importlib.import_module("21cmpy_gb300.schedule")
    cos = importlib.import_module("21cmpy_gb300.cosmology")
    lib_consts = importlib.import_module("21cmpy_gb300._lib")
    n, L, z = 512, 600.0, 7.5
    d = torch.from_numpy(grf.density_box(n, L, 0, z)).to(dev)
    st = sch.ionize_setup(n, L, z, zeta=40.0, t_vir_min=1e4, R_max=30.0, cosmo=cos.BASELINE_COSMO)
    c = cos.brightness_temperature_factor(z, cos.BASELINE_COSMO)
    edges = sch.pk_edges(n, L, NUM_BINS)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    with eng.ExcursionSetPlan(n, L, max_radii=64, device=dev) as plan:
        tuned = at.ensure_tuned(plan)
        xh, dT = torch.empty_like(d), torch.empty_like(d)

        def box():
            plan.run(d, st, out=xh)
            _, ave = plan.delta_T(xh, d, c, out=dT)
            plan.power_spectrum(dT, ave, edges)

        box()
        torch.cuda.synchronize(dev)
        e0, e1 = ev(), ev()
        e0.record()
        for _ in range(reps):
            box()
        e1.record()
        e1.synchronize()
        ms_box = e0.elapsed_time(e1) / reps
        # per pass, one box run serially (radii not overlapped) with an event pair per launch
        ov = plan.get_option(lib_consts.OPT_OVERLAP)
        plan.set_option(lib_consts.OPT_OVERLAP, 0)
        plan.profile_enable(4 * 64 + 32)
        box()
        torch.cuda.synchronize(dev)
        prof = plan.profile_read()
        plan.profile_enable(0)
        plan.set_option(lib_consts.OPT_OVERLAP, ov)
        half = 8.0 * (n // 2 + 1) / n
        bpv = {"col_z_inv_filter": 2 * half, "col_y_inv": 2 * half, "row_c2r_ionize": half + 8.0}
        passes = {}
        for k, b in bpv.items():
            ms, cnt = prof[k]
            us = 1e3 * ms / cnt
            gbs = b * n ** 3 / (us / 1e6) / 1e9
            passes[k] = {"us_per_launch": round(us, 2), "GB_s": round(gbs, 1), "frac": round(gbs / hbm_gbs, 3),
                         "algorithmic_bytes_per_voxel": round(b, 3)}

        # plain 3-D real FFTs: the engine's three passes against cuFFT through torch.fft
        def timed(fn, k=5):
            fn()
            torch.cuda.synchronize(dev)
            a, b = ev(), ev()
            a.record()
            for _ in range(k):
                fn()
            b.record()
            b.synchronize()
            return a.elapsed_time(b) / k

        X = plan.fft_r2c(d)
        ms_r2c = timed(lambda: plan.fft_r2c(d))
        ms_c2r = timed(lambda: plan.fft_c2r(X))
        ms_r2c_cufft = timed(lambda: torch.fft.rfftn(d))
        Xt = torch.fft.rfftn(d)
        ms_c2r_cufft = timed(lambda: torch.fft.irfftn(Xt, s=(n, n, n)))
        del X, Xt
    fft_bytes = (4.0 + half) * n ** 3              # read one array, write the other
    gb = lambda ms: round(fft_bytes / (ms / 1e3) / 1e9, 1)
    return {"workload": "one 512^3 box, BOX_LEN=600 Mpc, z=7.5, zeta=40, R_mfp=30 Mpc, Tvir=1e4 K, "
                        f"{st.n_radii} radii, delta_T + {NUM_BINS}-bin P(k)",
            "ms_per_box": ms_box, "value": n ** 3 * st.n_radii / (ms_box / 1e3), "unit": UNIT,
            "autotune": tuned.get("config"), "passes": passes,
            "passes_note": "one box run serially (radii not overlapped), CUDA event pair per launch",
            "fft_yardstick": {"engine_r2c_ms": ms_r2c, "engine_c2r_ms": ms_c2r, "cufft_r2c_ms": ms_r2c_cufft,
                              "cufft_c2r_ms": ms_c2r_cufft, "engine_r2c_GB_s": gb(ms_r2c), "engine_c2r_GB_s": gb(ms_c2r),
                              "cufft_r2c_GB_s": gb(ms_r2c_cufft), "cufft_c2r_GB_s": gb(ms_c2r_cufft),
                              "bytes_model": "4 B real + 8 (n/2+1)/n B half spectrum per voxel",
                              "note": "cuFFT (torch.fft) is timed as a yardstick only; it is not on any path"}}

def run_perturb(dev, hbm_gbs: float, reps: int = 20):
    """Zel'dovich move of a 512^3 initial-conditions box onto a 128^3 grid (the reference's default
    DIM / HII_DIM), inputs resident on the device; L2 is flushed between launches."""
    import numpy as np
    import torch
    pt = importlib.import_module("21cmpy_gb300.perturb")
    cos = importlib.import_module("21cmpy_gb300.cosmology")
    dim, sw = 512, 128
    g = torch.Generator(device=dev).manual_seed(3)
    d = torch.randn((dim,) * 3, device=dev, generator=g) * 1.5
    g0 = float(np.float32(cos.growth_factor(300.0, cos.PLANCK13)))
    ds = float(np.float32((cos.growth_factor(8.0, cos.PLANCK13) - g0) / 128.0))
    vs = [torch.randn((sw,) * 3, device=dev, generator=g) * (2.0 / sw / ds) for _ in range(3)]
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0.0
    with pt.PerturbPlan(dim, sw, device=dev) as plan:
        out = plan.move_mass(d, *vs, init_growth=g0, disp_scale=ds, mass_factor=64.0)
        for _ in range(3):
            plan.move_mass(d, *vs, init_growth=g0, disp_scale=ds, mass_factor=64.0, out=out)
        for _ in range(reps):
            flush.fill_(1.0)
            e0.record()
            plan.move_mass(d, *vs, init_growth=g0, disp_scale=ds, mass_factor=64.0, out=out)
            e1.record()
            e1.synchronize()
            total += e0.elapsed_time(e1)
    ms = total / reps
    # the velocity boxes at z = 8 from the same density (one 512^3 forward FFT, three inverse ones)
    ini = importlib.import_module("21cmpy_gb300.initial")
    scale = float(np.float32(cos.growth_rate(8.0, cos.PLANCK13))) / dim ** 3
    with ini.InitialConditions(dim, sw, 128.0, device=dev) as ic:
        for _ in range(2):
            ic.velocities(ic.plan.fft_r2c(d), scale)
        e0.record()
        for _ in range(5):
            ic.velocities(ic.plan.fft_r2c(d), scale)
        e1.record()
        e1.synchronize()
    vel_ms = e0.elapsed_time(e1) / 5
    # the oracle (float32 numpy restatement, one thread) on the first 64 DIM planes of the same input
    po = importlib.import_module("oracle.pf_oracle")
    dh = d[:64].cpu().numpy()
    vh = [v.cpu().numpy() for v in vs]
    t0 = time.perf_counter()
    po.move_mass(dh, *vh, g0, ds, 4.0, 64.0)
    cpu_s = time.perf_counter() - t0
    cpu_rate = dh.size / cpu_s
    # algorithmic bytes: read deltax once (4 B / DIM cell), the three displacement boxes and the
    # output once (16 B / HII cell), the accumulator cleared, summed into and read (24 B / HII cell)
    nbytes = 4.0 * dim ** 3 + 40.0 * sw ** 3
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"workload": "Zel'dovich move, DIM=512 -> HII_DIM=128, rms displacement 2 cells (pf_move_mass)",
            "ms": ms, "cells_per_s": dim ** 3 / (ms / 1e3),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_gbs, "unit": "GB/s", "frac": gbs / hbm_gbs,
                         "bytes_model": "4 B / DIM cell + 40 B / HII cell"},
            "l2": "flushed (256 MiB write) before every timed launch",
            "velocities_ms": vel_ms,
            "velocities_workload": "updated velocity boxes at z = 8 from the 512^3 density: forward 512^3 FFT, "
                                   "3 x (k-space shape, inverse 512^3 FFT, subsample to 128^3)",
            "cpu_baseline": {"value": cpu_rate, "unit": "cells/s", "cores": 1, "kind": "port",
                             "sample": f"64 of 512 DIM planes, numpy float32 oracle, one thread, {cpu_s:.1f} s"}}


def run_initial(dev, reps: int = 5):
    """Initial conditions for DIM = 512, HII_DIM = 128, BOX_LEN = 128 Mpc (the reference's defaults):
    spectrum, density, smoothed density and three displacement boxes (five 512^3 inverse FFTs)."""
    import torch
    ini = importlib.import_module("21cmpy_gb300.initial")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ini.InitialConditions(512, 128, 128.0, device=dev) as ic:
        normals = ic.normals(0)
        for _ in range(2):
            ic.generate(normals=normals)
        e0.record()
        for _ in range(reps):
            ic.generate(normals=normals)
        e1.record()
        e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return {"workload": "initial conditions DIM=512, HII_DIM=128, BOX_LEN=128 Mpc: density, smoothed density, "
                        "3 displacement boxes (5 inverse 512^3 FFTs), normals resident", "ms": ms}


def run_surrogate(dev, reps: int = 20):
    """Surrogate boxes/s: the network's forward pass on one 128^3 box (tcgen05 convolutions) next to
    the plain engine (forward FFT + all radii) on the same box, inputs resident on the device."""
    import torch
    S = importlib.import_module("21cmpy_gb300.surrogate")
    gen = S.DataGenerator(n=128, box_len=200.0, device=dev)
    params = dict(zeta=30.0, R_max=15.0, t_vir=1e4, z=8.0)
    s = gen.sample(5000, params)
    st = S.schedule.ionize_setup(gen.n, gen.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir, R_max=s.R_max,
                                 cosmo=gen.cosmo, table=gen.table)
    net = S.SurrogateNet(seed=0, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(3):
            fn()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    sg_ms = timed(lambda: net.forward(net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)))
    eng_ms = timed(lambda: gen.plan.run(s.delta, st))
    # one training step (forward keeping activations, backward with the weight gradients, Adam)
    opt = S.Adam(net.parameters(), lr=3e-4)

    def train_step():
        f = net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)
        pred, acts = net.forward(f, keep=True)
        dws, dbs = net.backward(acts, pred, s.xH)
        opt.step(dws + dbs, scale=1.0 / s.delta.numel())

    step_ms = timed(train_step)
    # the 32 -> 32 weight gradient alone (tensor cores at 128^3)
    n = gen.n
    xw = torch.randn((n, n, n, 32), device=dev).to(torch.bfloat16)
    dzw = torch.randn((n, n, n, 32), device=dev).to(torch.bfloat16)
    dw = torch.empty((27, 32, 32), device=dev)
    db = torch.empty(32, device=dev)
    wg_ms = timed(lambda: net._wgrad(n, 32, 32, xw, dzw, dw, db))
    net.check()
    flop = 2 * gen.n ** 3 * sum(27 * ci * co for ci, co in S.LAYERS)
    wg_flop = 2 * n ** 3 * 27 * 32 * 32
    gen.plan.close()
    return {"workload": "one 128^3 box, BOX_LEN=200 Mpc, z=8, zeta=30, R_mfp=15 Mpc, Tvir=1e4 K",
            "boxes_per_s": 1e3 / sg_ms, "ms_per_box": sg_ms, "tflops": flop / sg_ms / 1e9,
            "engine_boxes_per_s": 1e3 / eng_ms, "engine_ms_per_box": eng_ms,
            "ratio_surrogate_over_engine": eng_ms / sg_ms,
            "train_step_ms": step_ms, "wgrad_32x32_ms": wg_ms, "wgrad_32x32_tflops": wg_flop / wg_ms / 1e9,
            "note": "speed with random-init weights (it does not depend on them); accuracy of the trained "
                    "network against the plain engine is measured by Programs.train_surrogate"}


def run_batch(args, dev):
    """64 boxes of HII_DIM ~ U{64,96,128,160} with their own parameters, in one persistent launch
    (CUDA graph replay), against the same boxes looped through per-box plans."""
    import torch
    batch = importlib.import_module("21cmpy_gb300.batch")
    grf = importlib.import_module("21cmpy_gb300.grf")
    eng = importlib.import_module("21cmpy_gb300.engine")
    at = importlib.import_module("21cmpy_gb300.autotune")
    specs = grf.uneven_batch()
    boxes = batch.boxes_from_specs(specs, dev)
    stream = torch.cuda.current_stream(dev)
    b = batch.BatchedExcursionSet(boxes, use_graph=True, device=dev)
    sched_ms = at.tune_batch(b, schedules=[(0, 8), (0, 16), (32, 8)], repeats=2)
    for _ in range(3):
        b.run()
    b.check()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.run()
    e1.record(stream)
    e1.synchronize()
    b.check()
    t_batch = e0.elapsed_time(e1) / 1e3 / args.steps
    updates = b.voxel_radius_updates()
    info = b.info()
    # where the persistent launch's CTA time goes, per pass kind (one extra launch, counters on)
    b.profile(True)
    b.run()
    prof = b.profile_read()
    b.profile(False)
    total_cyc = sum(v["tile_cycles"] + v["wait_cycles"] for v in prof.values())
    op_share = {k: round((v["tile_cycles"] + v["wait_cycles"]) / total_cyc, 4) for k, v in prof.items()}
    cyc_per_tile = {k: round(v["tile_cycles"] / v["tiles"]) for k, v in prof.items()}
    b.close()
    plans = {}
    for d, st in boxes:
        if st.n not in plans:
            plans[st.n] = eng.ExcursionSetPlan(st.n, st.box_len, max_radii=64, device=dev)
            at.ensure_tuned(plans[st.n])
    outs = {n: torch.empty((n, n, n), dtype=torch.float32, device=dev) for n in plans}

    def loop():
        for d, st in boxes:
            plans[st.n].run(d, st, out=outs[st.n])
    for _ in range(2):
        loop()
    e0.record(stream)
    for _ in range(args.steps):
        loop()
    e1.record(stream)
    e1.synchronize()
    t_loop = e0.elapsed_time(e1) / 1e3 / args.steps
    for p in plans.values():
        p.close()
    # the same boxes through per-box plans on concurrent streams, captured into one CUDA graph
    g = batch.PlanGraphBatch(boxes, lanes=2, use_graph=True, device=dev)
    for _ in range(3):
        g.run()
    g.check()
    e0.record(stream)
    for _ in range(args.steps):
        g.run()
    e1.record(stream)
    e1.synchronize()
    g.check()
    t_graph = e0.elapsed_time(e1) / 1e3 / args.steps
    ginfo = g.info()
    g.close()
    modes = {"persistent": updates / t_batch, "plan_graph": updates / t_graph}
    best = max(modes, key=modes.get)
    return {"workload": "64 boxes, HII_DIM ~ U{64,96,128,160}, L = 1.5 N Mpc, zeta ~ U[10,80], "
                        "R_mfp ~ U[5,50] Mpc, log10 Tvir ~ U[4,5.3], z ~ U[6,10]; x_HI of every box",
            "value": modes[best], "mode": best, "unit": UNIT,
            "persistent_value": modes["persistent"], "persistent_ms_per_batch": 1e3 * t_batch,
            "persistent_schedule": {"lanes": info["lanes"], "tiles_per_ticket": info["chunk"],
                                    "tuned_ms": {f"{k[0]}x{k[1]}": round(v, 3) for k, v in sched_ms.items()}},
            "persistent_op_share": op_share, "persistent_cycles_per_tile": cyc_per_tile,
            "plan_graph_value": modes["plan_graph"], "plan_graph_ms_per_batch": 1e3 * t_graph,
            "per_box_plans_value": updates / t_loop, "per_box_plans_ms": 1e3 * t_loop,
            "launch": f"persistent: one launch per batch ({info['grid']} CTAs, {info['passes']} passes, "
                      f"{info['tiles']} tiles in {info['tickets']} tickets) replayed from a CUDA graph; plan_graph: {ginfo['lanes']} "
                      "autotuned plans on their own streams (two per box size, overlapped radii), the "
                      "whole batch captured in one CUDA graph; per_box_plans: one plan per size, boxes in turn"}


def measured_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if there is one."""
    path = os.path.join(ROOT, "profiles", "traffic_256.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and parts[0] == "traffic_bytes_per_launch" and parts[1] == kernel:
                    return float(parts[2])
    except OSError:
        pass
    return None


if __name__ == "__main__":
    sys.exit(main())
