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


def _boxes(specs):
    out = []
    for n, seed, z, zeta, rmax, tvir in specs:
        L = 1.5 * n
        d = torch.from_numpy(grf.density_box(n, L, seed, z)).cuda()
        st = sch.ionize_setup(n, L, z, zeta=zeta, t_vir_min=tvir, R_max=rmax, cosmo=cos.BASELINE_COSMO)
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
    assert info["passes"] == sum(4 + 3 * st.n_radii for _, st in boxes)
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
