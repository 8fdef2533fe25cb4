"""The persistent batched launch's work queue, built on the host (no device).

The queue is what makes one persistent launch safe: a CTA that takes a ticket may spin until the
ticket's dependencies are done, so every dependency must sit at an earlier ticket (held by a
resident CTA), and every buffer a pass writes must have no unfinished reader or writer.  Checked
for the uneven 64-box batch under every schedule the autotuner tries, in centre mode and with
every third box in sphere mode.
"""
import math

import pytest

from conftest import module

batch = module("batch")
grf = module("grf")
sch = module("schedule")
cos = module("cosmology")
at = module("autotune")


@pytest.fixture(scope="module")
def boxes():
    specs = grf.uneven_batch()
    nr = [sch.ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min, R_max=s.R_max,
                           cosmo=cos.BASELINE_COSMO).n_radii for s in specs]
    return [s.n for s in specs], nr


def _ancestors(q, k, memo):
    if k in memo:
        return memo[k]
    out = set()
    for d in (q[k]["dep"], q[k]["dep2"]):
        if d >= 0:
            out |= {d} | _ancestors(q, d, memo)
    memo[k] = out
    return out


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("lanes,chunk", at.BATCH_SCHEDULES)
def test_queue_is_ordered_complete_and_hazard_free(boxes, lanes, chunk, mixed):
    ns, nr = boxes
    upd = [int(mixed and i % 3 == 0) for i in range(len(ns))]
    pks = [int(mixed and i % 2 == 0) for i in range(len(ns))]
    q = batch.queue_plan(ns, nr, lanes, chunk, update=upd, pk=pks)
    assert len(q) == sum(5 + 3 * r + (r - 1 if u else 0) + 3 * k for r, u, k in zip(nr, upd, pks))
    # tickets: contiguous, chunk tiles each
    t = 0
    for d in q:
        assert d["first"] == t and d["tickets"] == math.ceil(d["tiles"] / chunk)
        t += d["tickets"]
    # each box's passes in its own order: forward, (z, y, row) per radius, final
    per_box = {}
    for k, d in enumerate(q):
        per_box.setdefault(d["box"], []).append(k)
    assert sorted(per_box) == list(range(len(ns)))
    memo = {}
    for b, ks in per_box.items():
        ops = [(q[k]["op"], q[k]["radius"]) for k in ks]
        per_r = lambda r: ("z_inv", "y_inv", "row_c2r") + (("paint",) if upd[b] and r >= 1 else ())  # noqa: E731
        want = [("wtab", 0), ("row_r2c", 0), ("y_fwd", 0), ("z_fwd", 0)] + \
            [(op, r) for r in range(nr[b]) for op in per_r(r)] + [("final", 0)] + \
            ([("pk_r2c", 0), ("y_fwd", 0), ("z_fwd_pk", 0)] if pks[b] else [])
        assert ops == want, b
        idx = {}
        for op_r, k in zip(ops, ks):
            idx.setdefault(op_r, k)             # the first y_fwd is the density's
        for k in ks:
            d = q[k]
            for dep in (d["dep"], d["dep2"]):
                assert dep < k and (dep < 0 or q[dep]["box"] == b)   # earlier ticket, same box
        # write-after-read / write-after-write on the two spectrum buffers: z_inv of radius r may
        # start only when radius r - 2's y and row passes (the last users of its buffer) are done
        for r in range(nr[b]):
            anc = _ancestors(q, idx[("z_inv", r)], memo)
            assert {idx[("z_fwd", 0)], idx[("wtab", 0)]} <= anc
            if r >= 2:
                assert {idx[("y_inv", r - 2)], idx[("row_c2r", r - 2)]} <= anc
            anc_y = _ancestors(q, idx[("y_inv", r)], memo)
            assert idx[("z_inv", r)] in anc_y
            anc_r = _ancestors(q, idx[("row_c2r", r)], memo)
            assert idx[("y_inv", r)] in anc_r
            if r >= 1:                     # threshold from radius r - 1, delta_R double buffer
                assert idx[("row_c2r", r - 1)] in anc_r
            if upd[b] and r >= 1:          # the painting reads the centres its row pass listed
                assert idx[("row_c2r", r)] in _ancestors(q, idx[("paint", r)], memo)
            if upd[b] and r >= 2:          # the list is refilled only after the last painting read it
                assert idx[("paint", r - 1)] in anc_r
        # the final step reads delta_R and every painted / flagged cell: all other passes are done
        i_fin = idx[("final", 0)]
        assert set(k for k in ks if k < i_fin) <= _ancestors(q, i_fin, memo)
        if pks[b]:                     # delta_T's transform reuses the forward spectrum's buffers
            chain = ks[ks.index(i_fin):]
            for later, earlier in zip(chain[1:], chain[:-1]):
                assert earlier in _ancestors(q, later, memo)


@pytest.mark.parametrize("lanes", [4, 8, 16])
def test_lanes_bound_the_boxes_in_flight(boxes, lanes):
    ns, nr = boxes
    q = batch.queue_plan(ns, nr, lanes, 1)
    last = {}
    for k, d in enumerate(q):
        last[d["box"]] = k
    open_boxes, peak = set(), 0
    for k, d in enumerate(q):
        open_boxes.add(d["box"])
        peak = max(peak, len(open_boxes))
        if last[d["box"]] == k:
            open_boxes.discard(d["box"])
    assert peak == lanes


def test_lanes_are_balanced_by_voxel_radius_work(boxes):
    ns, nr = boxes
    lanes = 8
    q = batch.queue_plan(ns, nr, lanes, 1)
    # recover the lanes: a box opens when an earlier one closes (or at the start)
    order = []
    for d in q:
        if d["box"] not in order:
            order.append(d["box"])
    cost = [n ** 3 * r for n, r in zip(ns, nr)]
    first_wave = order[:lanes]
    heaviest = sorted(range(len(ns)), key=lambda i: -cost[i])[:lanes]
    assert sorted(first_wave) == sorted(heaviest)


def test_queue_rejects_bad_input():
    _lib = module("_lib")
    with pytest.raises(_lib.EngineError):
        batch.queue_plan([100], [4])
    with pytest.raises(_lib.EngineError):
        batch.queue_plan([64], [4], chunk=0)
