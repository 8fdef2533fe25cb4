"""Tile-shape and radix-schedule autotuner for the engine's FFT passes.

For a box size it times, on the device, every combination of the TMA passes' tile shapes
(``ES_OPT_COL_TILE`` x ``ES_OPT_ROW_TILE``) and of the per-radius passes' radix schedules
(``ES_OPT_COL_RADIX`` x ``ES_OPT_ROW_RADIX``: radices up to 16, or up to 8 with one more stage),
plus the synchronous-tile passes, running one whole box through the path (forward transform,
every radius, final step, delta_T and P(k)), and keeps the fastest.  A second stage times, on the
best of those, the overlapped-radius schedules (``ES_OPT_OVERLAP`` with per-SM CTA caps
``ES_OPT_ROW_CTAS`` / ``ES_OPT_COL_CTAS``), then the runner-up tile shapes with the best schedule.  Results are cached per GPU model, box size and library version in a JSON file
(``$ES_AUTOTUNE_CACHE`` or ``~/.cache/21cmpy_gb300/autotune.json``), so later plans of the same
size start tuned.

``tune_batch`` is the persistent batched launch's stage: it times the work-queue schedules
(``es_batch_set_schedule``: boxes in flight x tiles per ticket) on the batch itself and keeps the
fastest.
"""
from __future__ import annotations

import json
import os
import threading
from pathlib import Path

import numpy as np
import torch

from . import _lib, cosmology, schedule

# (variant, col tile, row tile, col radix schedule, row radix schedule)
CANDIDATES = [(1, c, r, cr, rr) for c in range(3) for r in range(4) for cr in range(2) for rr in range(2)] + \
    [(0, 0, 0, 0, 0)]
# (overlap, row-pass CTAs per SM, column-pass CTAs per SM), appended to a tile configuration
OVERLAP = [(0, 0, 0), (1, 0, 0), (1, 1, 1), (1, 1, 2), (1, 1, 3), (1, 2, 1), (1, 2, 2)]


def with_overlap(config, ov) -> tuple:
    return tuple(config)[:5] + tuple(ov)
_lock = threading.Lock()


def cache_path() -> Path:
    p = os.environ.get("ES_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "21cmpy_gb300" / "autotune.json"


def _key(device, n: int) -> str:
    lib = _lib.load()
    return f"{torch.cuda.get_device_name(device)}|n={n}|v={lib.es_version()}"


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(table: dict):
    path = cache_path()
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass                     # a read-only home only costs re-tuning


def apply(plan, config) -> None:
    config = tuple(config) + (0,) * max(0, 8 - len(config))    # entries without later options
    variant, col_tile, row_tile, col_radix, row_radix, overlap, row_ctas, col_ctas = config[:8]
    plan.set_option(_lib.OPT_COL_VARIANT, variant)
    plan.set_option(_lib.OPT_COL_TILE, col_tile)
    plan.set_option(_lib.OPT_ROW_TILE, row_tile)
    plan.set_option(_lib.OPT_COL_RADIX, col_radix)
    plan.set_option(_lib.OPT_ROW_RADIX, row_radix)
    plan.set_option(_lib.OPT_OVERLAP, overlap)
    plan.set_option(_lib.OPT_ROW_CTAS, row_ctas)
    plan.set_option(_lib.OPT_COL_CTAS, col_ctas)


def cached(device, n: int):
    entry = _load().get(_key(device, n))
    return tuple(entry["config"]) if entry else None


def tune(plan, repeats: int = 3, store: bool = True) -> dict:
    """Time every candidate on `plan`'s box size and apply the fastest; returns the timings."""
    from .grf import density_box
    n, L = plan.n, plan.box_len
    dev = plan.device
    with torch.cuda.device(dev):
        d = torch.from_numpy(density_box(n, L, seed=12345, z=8.0)).to(dev)
        cosmo = cosmology.BASELINE_COSMO
        R_max = min(15.0, 0.2 * L)
        st = schedule.ionize_setup(n, L, 8.0, zeta=30.0, t_vir_min=1e4, R_max=R_max, cosmo=cosmo)
        st.steps = st.steps[: plan.max_radii]
        c = cosmology.brightness_temperature_factor(8.0, cosmo)
        edges = schedule.pk_edges(n, L, 20)
        xh = torch.empty_like(d)
        dT = torch.empty_like(d)
        stream = torch.cuda.current_stream(dev)
        times = {}

        def box():
            plan.run(d, st, out=xh)
            _, ave = plan.delta_T(xh, d, c, out=dT)
            plan.power_spectrum(dT, ave, edges)

        def time_config(cfg):
            apply(plan, cfg)
            box()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(repeats):
                box()
            e1.record(stream)
            e1.synchronize()
            times[tuple(cfg)] = e0.elapsed_time(e1) / repeats

        for cfg in CANDIDATES:
            time_config(with_overlap(cfg, OVERLAP[0]))
        ranked = sorted(times, key=times.get)
        for ov in OVERLAP[1:]:
            time_config(with_overlap(ranked[0], ov))
        best_ov = min(times, key=times.get)[5:]
        for cfg in ranked[1:3]:
            if with_overlap(cfg, best_ov) not in times:
                time_config(with_overlap(cfg, best_ov))
        plan.check()
        best = min(times, key=times.get)
        apply(plan, best)
    result = {"config": list(best), "ms_per_box": times[best],
              "candidates": {"/".join(map(str, cfg)): round(ms, 4) for cfg, ms in times.items()}}
    if store:
        with _lock:
            table = _load()
            table[_key(dev, n)] = result
            _store(table)
    return result


def ensure_tuned(plan, allow_tuning: bool = True):
    """Apply the cached configuration for this plan's size, tuning first if there is none."""
    cfg = cached(plan.device, plan.n)
    if cfg is not None:
        apply(plan, cfg)
        return {"config": list(cfg), "source": "cache"}
    if not allow_tuning:
        return {"config": None, "source": "default"}
    r = tune(plan)
    r["source"] = "tuned"
    return r


# (lanes, tiles per ticket) of the persistent batched launch; lanes 0 = every box its own lane
BATCH_SCHEDULES = [(0, 8), (0, 16), (0, 4), (32, 8), (16, 8), (8, 16)]


def tune_batch(b, schedules=BATCH_SCHEDULES, repeats: int = 3) -> dict:
    """Time every schedule on the batch ``b`` (a ``BatchedExcursionSet``), replaying its graph,
    and leave the fastest set; returns {schedule: ms per batch}."""
    dev = b.device
    stream = torch.cuda.current_stream(dev)
    times = {}
    for lanes, chunk in schedules:
        b.set_schedule(lanes, chunk)
        b.run()
        b.run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            b.run()
        e1.record(stream)
        e1.synchronize()
        b.check()
        times[(lanes, chunk)] = e0.elapsed_time(e1) / repeats
    best = min(times, key=times.get)
    b.set_schedule(*best)
    return times
