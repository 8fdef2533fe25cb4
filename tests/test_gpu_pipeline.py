"""The pipelined sweep API against box-by-box simulate_box (GPU)."""
import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pipe():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("Programs.pipeline")


def test_sweep_equals_box_by_box(pipe):
    grf = module("grf")
    cos = module("cosmology")
    n, L = 64, 100.0
    zs = [7.0, 8.5, 10.0, 9.0, 6.5]
    boxes = [grf.density_box(n, L, seed, z, cosmo=cos.BASELINE_COSMO).astype(np.float32) for seed, z in enumerate(zs)]
    params = {"ZETA": 30.0, "ION_Tvir_MIN": 1e4, "R_BUBBLE_MAX": 15.0, "COSMO": cos.BASELINE_COSMO, "NUM_BINS": 12}
    pd = {"BoxSize": L, "HIIdim": n}
    sweep = pipe.simulate_sweep([torch.from_numpy(b).pin_memory() for b in boxes], pd, zs, fil=0, params=params)
    for b, z, r in zip(boxes, zs, sweep):
        one = pipe.simulate_box(b, pd, Z=z, fil=0, params=params)
        assert np.array_equal(r["xH"].numpy(), one["xH"])
        assert np.array_equal(r["dT"].numpy(), one["dT"])
        assert r["nf"] == one["nf"] and r["ave"] == one["ave"] and r["n_radii"] == one["n_radii"]
        assert np.array_equal(r["ps_ave"], one["ps_ave"]) and np.array_equal(r["k_ave"], one["k_ave"])
        assert np.array_equal(r["count"], one["count"])
