"""Failure detection of the per-plan TMA passes, without a GPU fault.

A debug option makes CTA 0 of one pass announce 16 bytes more than its first tile brings, so
that tile's wait can only end by running out (the copies themselves land normally).  The
bounded wait gives up, the CTA waits (bounded again) for the copies it issued, records the
error word and leaves; the host reads ES_E_DEVICE from es_plan_check and the same plan then
reproduces its earlier results bit for bit.
"""
import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

cos = module("cosmology")
sch = module("schedule")
grf = module("grf")


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return module("engine")


@pytest.mark.parametrize("overlap", [0, 1])
@pytest.mark.parametrize("stall", ["col_z", "row_c2r", "row_r2c"])
def test_timed_out_tile_wait_reports_and_plan_recovers(eng, stall, overlap):
    _lib = module("_lib")
    code = {"col_z": _lib.STALL_COL_Z_INV, "row_c2r": _lib.STALL_ROW_C2R, "row_r2c": _lib.STALL_ROW_R2C}[stall]
    n, L, z = 64, 100.0, 8.0
    d = torch.from_numpy(grf.density_box(n, L, seed=2, z=z)).cuda()
    st = sch.ionize_setup(n, L, z, zeta=30.0, t_vir_min=1e4, R_max=15.0, cosmo=cos.BASELINE_COSMO)
    with eng.ExcursionSetPlan(n, L) as p:
        p.set_option(_lib.OPT_OVERLAP, overlap)
        good, good_nf = p.run(d, st)
        good, good_nf = good.clone(), good_nf.clone()
        p.check()
        p.set_option(_lib.OPT_WAIT_LOG2, 12)
        p.set_option(_lib.OPT_DEBUG_STALL, code)
        assert p.get_option(_lib.OPT_DEBUG_STALL) == code
        p.run(d, st)
        with pytest.raises(_lib.EngineError) as ei:
            p.check()
        assert ei.value.code == _lib.ES_E_DEVICE
        p.set_option(_lib.OPT_DEBUG_STALL, 0)
        p.set_option(_lib.OPT_WAIT_LOG2, 0)
        again, again_nf = p.run(d, st)
        p.check()                       # the error word was cleared by the failed check
        assert torch.equal(again, good)
        assert torch.equal(again_nf, good_nf)
        assert np.isfinite(again_nf.item())


def test_wait_and_stall_options_are_validated(eng):
    _lib = module("_lib")
    with eng.ExcursionSetPlan(32, 48.0) as p:
        for opt, bad in ((_lib.OPT_WAIT_LOG2, 5), (_lib.OPT_WAIT_LOG2, 31), (_lib.OPT_DEBUG_STALL, 4),
                         (_lib.OPT_DEBUG_STALL, -1)):
            with pytest.raises(_lib.EngineError):
                p.set_option(opt, bad)
        assert p.get_option(_lib.OPT_WAIT_LOG2) == 0
        assert p.get_option(_lib.OPT_DEBUG_STALL) == 0
