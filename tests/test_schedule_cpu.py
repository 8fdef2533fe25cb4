"""CPU checks of the host-side scheduling logic: autotuner configurations, sweep lane slots and
the bench line's roofline figures."""
import importlib.util
import os

import pytest

from conftest import module

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _FakePlan:
    def __init__(self):
        self.options = {}

    def set_option(self, option, value):
        self.options[option] = value


def test_autotune_configurations():
    at = module("autotune")
    _lib = module("_lib")
    # every candidate names (variant, column tile, row tile, column radix, row radix)
    assert len(set(at.CANDIDATES)) == len(at.CANDIDATES) == 3 * 4 * 2 * 2 + 1
    assert all(len(c) == 5 for c in at.CANDIDATES)
    assert at.OVERLAP[0] == (0, 0, 0) and all(o[0] == 1 for o in at.OVERLAP[1:])
    assert at.with_overlap((1, 2, 3, 0, 1, 9, 9, 9), (1, 1, 2)) == (1, 2, 3, 0, 1, 1, 1, 2)
    # older cache entries without radix schedules or overlap settings run with those off
    p = _FakePlan()
    at.apply(p, (1, 1, 3))
    assert p.options == {_lib.OPT_COL_VARIANT: 1, _lib.OPT_COL_TILE: 1, _lib.OPT_ROW_TILE: 3,
                         _lib.OPT_COL_RADIX: 0, _lib.OPT_ROW_RADIX: 0, _lib.OPT_OVERLAP: 0,
                         _lib.OPT_ROW_CTAS: 0, _lib.OPT_COL_CTAS: 0}
    at.apply(p, [1, 1, 3, 0, 0, 1, 2, 2])
    assert (p.options[_lib.OPT_OVERLAP], p.options[_lib.OPT_ROW_CTAS], p.options[_lib.OPT_COL_CTAS]) == (1, 2, 2)


@pytest.mark.parametrize("lanes", [1, 2, 3, 4])
def test_sweep_slots_are_reused_only_two_boxes_later(lanes):
    # a lane runs its boxes in turn; a box may still be copied in, computed or copied out while the
    # lane's next box starts, so its slot must not come back before the box after that
    pipe = module("Programs.pipeline")
    seen = {}
    for i in range(12 * lanes):
        lane, slot = pipe.lane_slot(i, lanes)
        assert lane == i % lanes and 0 <= slot < 2 * lanes and slot // 2 == lane
        if slot in seen:
            assert i - seen[slot] == 2 * lanes
        seen[slot] = i
    assert len(seen) == 2 * lanes


def test_bench_roofline_line():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    prof = {"row_c2r_ionize": (20.0, 100), "col_z_inv_filter": (15.0, 100), "col_y_inv": (15.0, 100)}
    b = 200e6
    # serial schedule: the event-bracketed rate is the kernel's own
    line = bench.roofline_line("row_c2r_ionize", b, 20.0, 100, b * 100 / 0.02 / 1e9, 6000.0, "measured", None,
                               None, prof, 0.05, 1)
    assert line["achieved"] == pytest.approx(1000.0) and line["frac"] == pytest.approx(1000.0 / 6000.0)
    # concurrent schedule: the kernel alone leads, live and apportioned figures beside it
    iso = {"achieved": 3000.0, "frac": 0.5, "launch_ms": 0.0667}
    line = bench.roofline_line("row_c2r_ionize", b, 20.0, 100, 1000.0, 6000.0, "measured", None, iso, prof, 0.03, 1)
    assert line["achieved"] == 3000.0 and line["live"]["achieved"] == pytest.approx(1000.0)
    app = line["apportioned"]
    assert app["share_of_event_time"] == pytest.approx(0.4)
    assert app["launch_ms"] == pytest.approx(1e3 * 0.03 * 0.4 / 100)
    assert app["achieved"] == pytest.approx(b / (app["launch_ms"] / 1e3) / 1e9)


def test_sweep_argument_checks_come_first():
    # bad arguments are reported before any device work (here there is no device at all)
    pipe = module("Programs.pipeline")
    import numpy as np
    box = np.zeros((8, 8, 8), np.float32)
    with pytest.raises(ValueError, match="lanes"):
        pipe.simulate_sweep([box], {"BoxSize": 12.0}, [8.0], lanes=0)
    with pytest.raises(ValueError, match="redshift"):
        pipe.simulate_sweep([box, box], {"BoxSize": 12.0}, [8.0])
    assert pipe.simulate_sweep([], {"BoxSize": 12.0}, []) == []


def test_lane_plans_fit_the_plan_cache():
    pipe = module("Programs.pipeline")
    common = module("Programs._common")
    # every lane of a sweep keeps its plan cached while a plan of another size stays cached too
    assert common.MAX_CACHED_PLANS >= 2 * pipe.MAX_LANES
