"""The batched persistent engine against the per-box engine and the oracle (GPU)."""
import ctypes as C

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import es_oracle as O  # noqa: E402

cos = module("cosmology")
sch = module("schedule")
grf = module("grf")
PARTIAL_ATOL = 2e-4


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("engine"), module("batch")


def _boxes(specs, **kw):
    out = []
    for n, seed, z, zeta, rmax, tvir, *extra in specs:
        L = 1.5 * n
        d = torch.from_numpy(grf.density_box(n, L, seed, z)).cuda()
        args = dict(kw)
        if extra:
            args.update(extra[0])
        st = sch.ionize_setup(n, L, z, zeta=zeta, t_vir_min=tvir, R_max=rmax, cosmo=cos.BASELINE_COSMO, **args)
        out.append((d, st))
    return out


SPECS = [(32, 1, 7.0, 30.0, 10.0, 1e4), (48, 2, 8.5, 55.0, 20.0, 3e4), (64, 3, 6.5, 12.0, 6.0, 1e4),
         (96, 4, 9.0, 70.0, 40.0, 1e5), (64, 5, 7.5, 30.0, 15.0, 2e4), (32, 6, 6.2, 80.0, 48.0, 1.5e4),
         (128, 7, 8.0, 25.0, 12.0, 1e4), (48, 8, 10.0, 45.0, 30.0, 5e4)]


def test_batch_matches_per_box_engine_and_oracle(mods):
    eng, batch = mods
    boxes = _boxes(SPECS)
    with batch.BatchedExcursionSet(boxes, use_graph=True) as b:
        outs, nf = b.run()
        b.check()
        outs = [o.clone() for o in outs]
        nf = nf.clone()
        info = b.info()
    assert info["passes"] == sum(5 + 3 * st.n_radii for _, st in boxes)
    for i, (d, st) in enumerate(boxes):
        with eng.ExcursionSetPlan(st.n, st.box_len) as p:
            xh, nfp = p.run(d, st)
        diff = (outs[i] - xh).abs()
        assert (diff > PARTIAL_ATOL).float().mean().item() <= 1e-5, (i, diff.max().item())
        assert abs(nf[i].item() - nfp.item()) <= 1e-5, i
    for i in (0, 2):                      # two boxes straight against the float64 oracle
        d, st = boxes[i]
        ref = O.conv_bubbles(d.cpu().numpy(), st)
        ion = 1.0 - outs[i].cpu().numpy().astype(np.float64)
        bad = (np.abs(ion - ref["ionized"]) > PARTIAL_ATOL) & ~ref["exempt"]
        assert bad.sum() == 0, i


SPHERE_SPECS = [(64, 11, 8.0, 30.0, 10.0, 1e4, dict(update=1)), (48, 12, 7.5, 50.0, 20.0, 2e4),
                (96, 13, 8.5, 40.0, 15.0, 1e4, dict(update=1)),
                (64, 14, 8.0, 30.0, 8.0, 1e4, dict(update=1, ref_compat=True)),
                (32, 15, 9.0, 60.0, 30.0, 3e4, dict(update=1, filter_type=2))]


def test_batch_sphere_painting_matches_per_box_engine(mods):
    # sphere mode (find_bubbles.cu:73-140) in the persistent launch, mixed with a centre-mode box:
    # the row pass lists the centres, a painting pass per radius marks their balls
    eng, batch = mods
    boxes = _boxes(SPHERE_SPECS)
    assert [st.update for _, st in boxes] == [1, 0, 1, 1, 1]
    with batch.BatchedExcursionSet(boxes, use_graph=True, lanes=2, chunk=4) as b:
        outs, nf = b.run()
        b.check()
        outs = [o.clone() for o in outs]
        nf = nf.clone()
        info = b.info()
    assert info["passes"] == sum(5 + 3 * st.n_radii + (st.n_radii - 1 if st.update else 0) for _, st in boxes)
    for i, (d, st) in enumerate(boxes):
        with eng.ExcursionSetPlan(st.n, st.box_len) as p:
            xh, nfp = p.run(d, st)
        diff = (outs[i] - xh).abs()
        assert (diff > PARTIAL_ATOL).float().mean().item() <= 1e-5, (i, diff.max().item())
        assert abs(nf[i].item() - nfp.item()) <= 1e-5, i
    d, st = boxes[0]                       # one sphere box straight against the float64 oracle
    ref = O.conv_bubbles(d.cpu().numpy(), st)
    ion = 1.0 - outs[0].cpu().numpy().astype(np.float64)
    bad = (np.abs(ion - ref["ionized"]) > PARTIAL_ATOL) & ~ref["exempt"]
    assert bad.sum() == 0
    assert ref["flags"].mean() > 0.02     # the painting does real work here


def test_batch_delta_T_and_pk_match_per_box_plans(mods):
    # delta_T (fused into the final step) and P(k) (delta_T's forward transform ending in the
    # binning z pass) inside the persistent launch, for some boxes of a mixed batch, against the
    # per-box plan's es_delta_T / es_power_spectrum and against the float64 oracle's P(k)
    eng, batch = mods
    boxes = _boxes(SPECS[:4] + SPHERE_SPECS[:1])
    facs = [cos.brightness_temperature_factor(st.z, cos.BASELINE_COSMO) for _, st in boxes]
    edges = [sch.pk_edges(st.n, st.box_len, 12 + i) for i, (_, st) in enumerate(boxes)]
    with batch.BatchedExcursionSet(boxes, use_graph=True, lanes=3, chunk=4, t_factors=facs, pk_edges=edges) as b:
        outs, nf = b.run()
        b.check()
        outs = [o.clone() for o in outs]
        dT = [t.clone() for t in b.dT]
        ave = b.ave.clone()
        pk = [q.cpu().numpy() for q in b.pk]
        b.run()                                  # a replay gives the same products
        b.check()
        assert all(torch.equal(x, y) for x, y in zip(dT, b.dT)) and torch.equal(ave, b.ave)
        assert all(np.array_equal(x, y.cpu().numpy()) for x, y in zip(pk, b.pk))
    for i, (d, st) in enumerate(boxes):
        with eng.ExcursionSetPlan(st.n, st.box_len) as p:
            xh, _ = p.run(d, st)
            t, a = p.delta_T(xh, d, facs[i])
            q = p.power_spectrum(t, a, edges[i]).cpu().numpy()
        # delta_T is c x_HI (1 + delta) of the batch's own x_HI, and close to the plan's
        own = np.float32(facs[i]) * outs[i].cpu().numpy() * (np.float32(1) + d.cpu().numpy())
        assert np.allclose(dT[i].cpu().numpy(), own, rtol=1e-6, atol=0), i
        assert ((dT[i] - t).abs() > PARTIAL_ATOL * abs(facs[i]) * 2).float().mean().item() <= 1e-5, i
        assert abs(ave[i].item() - a.item()) <= 1e-5 * abs(a.item()), i
        assert np.array_equal(pk[i][2], q[2]), i          # exact mode counts
        nz = q[2] > 0
        assert np.allclose(pk[i][1][nz], q[1][nz], rtol=1e-5), i
        assert (np.abs(pk[i][0][nz] - q[0][nz]) / np.abs(q[0][nz])).max() <= 1e-4, i
    # one box's P(k) against the float64 oracle on the batch's own delta_T
    from parity_util import compare_pk
    d, st = boxes[1]
    dT_o, ave_o = O.delta_T(outs[1].cpu().numpy().astype(np.float64), d.cpu().numpy(), facs[1])
    compare_pk(pk[1], O.power_spectrum(dT_o, ave_o, st.box_len, edges[1]), "batch P(k)")


def test_batch_profile_counts_every_tile(mods):
    _, batch = mods
    boxes = _boxes(SPECS[:3])
    with batch.BatchedExcursionSet(boxes, use_graph=True, chunk=4) as b:
        b.profile(True)
        b.run()
        b.run()
        prof = b.profile_read()
        b.profile(False)
        b.check()
    q = batch.queue_plan([st.n for _, st in boxes], [st.n_radii for _, st in boxes], 0, 4)
    for op in ("z_inv", "y_inv", "row_c2r", "final", "wtab"):
        assert prof[op]["tiles"] == 2 * sum(d["tiles"] for d in q if d["op"] == op), op
        assert prof[op]["tickets"] == 2 * sum(d["tickets"] for d in q if d["op"] == op), op
        assert prof[op]["tile_cycles"] > 0


def test_batch_graph_replay_is_deterministic(mods):
    _, batch = mods
    boxes = _boxes(SPECS[:4])
    with batch.BatchedExcursionSet(boxes, use_graph=True) as b:
        o1, n1 = b.run()
        r1 = [o.clone() for o in o1], n1.clone()
        o2, n2 = b.run()
        b.check()
        assert all(torch.equal(a, c) for a, c in zip(r1[0], o2))
        assert torch.equal(r1[1], n2)


def test_batch_schedules_give_identical_results(mods):
    # the queue order changes which CTA runs a tile and when, not what a tile computes or the
    # fixed order of its reductions: every schedule gives the same bits
    _, batch = mods
    at = module("autotune")
    boxes = _boxes(SPECS)
    ref = None
    with batch.BatchedExcursionSet(boxes, use_graph=True) as b:
        for lanes, chunk in [(0, 1), (4, 1), (8, 2), (2, 4), (3, 64)]:
            b.set_schedule(lanes, chunk)
            assert b.schedule()["lanes"] == lanes and b.schedule()["chunk"] == chunk
            outs, nf = b.run()
            b.check()
            got = [o.clone() for o in outs], nf.clone()
            if ref is None:
                ref = got
            else:
                assert all(torch.equal(a, c) for a, c in zip(ref[0], got[0])), (lanes, chunk)
                assert torch.equal(ref[1], got[1])
        times = at.tune_batch(b, schedules=[(0, 1), (4, 2)], repeats=1)
        assert set(times) == {(0, 1), (4, 2)}
        best = min(times, key=times.get)
        assert (b.schedule()["lanes"], b.schedule()["chunk"]) == best
        outs, nf = b.run()
        b.check()
        assert all(torch.equal(a, c) for a, c in zip(ref[0], outs))


def test_batch_stalled_dependency_aborts_and_reports(mods):
    # failure detection without a GPU fault: one pass waits for a tile that never comes; its
    # bounded wait runs out, the launch aborts, the host reads the error and the device stays usable
    _, batch = mods
    _lib = module("_lib")
    boxes = _boxes(SPECS[:3])
    b = batch.BatchedExcursionSet(boxes, use_graph=False)
    try:
        rc = b.lib.es_batch_debug_stall(b.handle, 7, 20000)
        _lib.check("es_batch_debug_stall", rc, b.lib)
        b.run()
        with pytest.raises(_lib.EngineError) as ei:
            b.check()
        assert ei.value.code == -5
    finally:
        b.close()
    with batch.BatchedExcursionSet(_boxes(SPECS[:2]), use_graph=False) as ok:
        ok.run()
        ok.check()
        assert torch.isfinite(ok.nf).all()


@pytest.mark.parametrize("overlap", [0, 1])
def test_plan_graph_batch_matches_per_box_plans(mods, overlap):
    # per-box plans on concurrent streams, captured in one CUDA graph and replayed twice, give the
    # per-box plan's outputs bit for bit (same kernels, same grids, same reduction order)
    eng, batch = mods
    _lib = module("_lib")
    boxes = _boxes(SPECS)
    with batch.PlanGraphBatch(boxes, lanes=2, use_graph=True, tune=False) as g:
        for _p, _s, _idx in g.lanes:
            _p.set_option(_lib.OPT_OVERLAP, overlap)
        g.run()
        outs, nf = g.run()
        g.check()
        outs = [o.clone() for o in outs]
        nf = nf.clone()
        assert g.info()["lanes"] == sum(min(2, sum(1 for _, s in boxes if (s.n, s.box_len) == k))
                                        for k in {(s.n, s.box_len) for _, s in boxes})
    for i, (d, st) in enumerate(boxes):
        with eng.ExcursionSetPlan(st.n, st.box_len) as p:
            p.set_option(_lib.OPT_OVERLAP, overlap)
            xh, nfp = p.run(d, st)
        assert torch.equal(outs[i], xh), i
        assert nf[i].item() == nfp.item(), i
