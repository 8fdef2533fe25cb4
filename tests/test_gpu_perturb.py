"""The density evolution (perturb_field) on the GPU against its CPU restatement (GPU)."""
import os

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import pf_oracle as PO  # noqa: E402

cos = module("cosmology")


@pytest.fixture(scope="module")
def pt():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("perturb")


def _inputs(dim, sw, seed, cells):
    """Gaussian deltax at z = 0 and displacement boxes whose rms move is `cells` HII cells at z = 8."""
    rng = np.random.default_rng(seed)
    delta = (rng.standard_normal((dim,) * 3) * 1.5).astype(np.float32)
    g = np.float32(cos.growth_factor(8.0, cos.PLANCK13))
    g0 = np.float32(cos.growth_factor(300.0, cos.PLANCK13))
    L = np.float32(100.0)
    ds = np.float32((g - g0) / L)
    v = [(rng.standard_normal((sw,) * 3) * (cells / sw / float(ds))).astype(np.float32) for _ in range(3)]
    return delta, v, g0, ds


@pytest.mark.parametrize("dim,sw,cells", [(64, 32, 1.5), (128, 32, 3.0), (96, 32, 0.7), (100, 64, 2.0), (64, 64, 5.0)])
def test_move_mass_is_bit_exact(pt, dim, sw, cells):
    delta, v, g0, ds = _inputs(dim, sw, dim + sw, cells)
    pf = np.float32(dim) / np.float32(sw)
    mf = np.float32(pf ** 3.0)
    ref = PO.move_mass(delta, *v, g0, ds, pf, mf)
    with pt.PerturbPlan(dim, sw, pixel_factor=float(pf)) as plan:
        d = torch.from_numpy(delta).cuda()
        vs = [torch.from_numpy(x).cuda() for x in v]
        out = plan.move_mass(d, *vs, init_growth=float(g0), disp_scale=float(ds), mass_factor=float(mf))
        got = out.cpu().numpy()
        again = plan.move_mass(d, *vs, init_growth=float(g0), disp_scale=float(ds), mass_factor=float(mf)).cpu().numpy()
    assert np.array_equal(got, ref), np.abs(got - ref).max()
    assert np.array_equal(again, got)                 # order-independent integer sums


def test_move_mass_full_size_conserves_mass(pt):
    # the reference's default sizes: DIM = 512 onto HII_DIM = 128; mean of (updated + 1) * MASS_FACTOR
    # over the HII grid equals the mean mass of the DIM^3 cells, and two runs agree bit for bit
    dim, sw = 512, 128
    g = torch.Generator(device="cuda").manual_seed(5)
    d = torch.randn((dim,) * 3, device="cuda", generator=g) * 1.5
    ds = float(np.float32((cos.growth_factor(8.0, cos.PLANCK13) - cos.growth_factor(300.0, cos.PLANCK13)) / 128.0))
    vs = [torch.randn((sw,) * 3, device="cuda", generator=g) * (2.0 / sw / ds) for _ in range(3)]
    g0 = float(np.float32(cos.growth_factor(300.0, cos.PLANCK13)))
    with pt.PerturbPlan(dim, sw) as plan:
        a = plan.move_mass(d, *vs, init_growth=g0, disp_scale=ds, mass_factor=64.0)
        b = plan.move_mass(d, *vs, init_growth=g0, disp_scale=ds, mass_factor=64.0)
    assert torch.equal(a, b)
    mass = (1.0 + np.float32(g0) * d.double()).mean().item()
    assert abs((a.double() + 1.0).mean().item() - mass) < 1e-6
    assert torch.isfinite(a).all()


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim,sw,ref_compat", [(64, 32, False), (128, 64, True), (256, 128, False)])
def test_velocities_match_float64_restatement(pt, dim, sw, ref_compat):
    L = 1.5 * dim
    rng = np.random.default_rng(dim)
    delta = (rng.standard_normal((dim,) * 3) * 1.5).astype(np.float32)
    rate = np.float32(cos.growth_rate(9.0, cos.PLANCK13))
    pf = np.float32(dim) / np.float32(sw)
    R = float(np.float32(np.float32(0.620350491) * np.float32(L) / np.float32(sw)))
    got = pt.updated_velocities(torch.from_numpy(delta).cuda(), sw, L, float(rate), pixel_factor=float(pf),
                                ref_compat=ref_compat)
    ref = PO.velocities(delta, sw, L, R, rate, pf, ref_compat=ref_compat)
    for name in ("vx", "vy", "vz"):
        assert _rel(got[name].cpu().numpy(), ref[name]) < 2e-5, name


def test_evolve_linear_is_bit_exact(pt):
    rng = np.random.default_rng(7)
    x = rng.standard_normal((64,) * 3).astype(np.float32)
    out = pt.evolve_linear(torch.from_numpy(x).cuda(), 0.1234).cpu().numpy()
    assert np.array_equal(out, PO.evolve_linear(x, np.float32(0.1234)))


def test_drop_in_program_reads_and_writes_reference_files(pt, tmp_path):
    prog = module("Programs.perturb_field")
    boxes = tmp_path / "Boxes"
    boxes.mkdir()
    dim, sw, L = 64, 32, 100.0
    delta, v, g0, ds = _inputs(dim, sw, 11, 1.0)
    np.save(boxes / "deltax_z0.00_64_100Mpc.npy", delta)
    for name, arr in zip("xyz", v):
        np.save(boxes / f"v{name}overddot_32_100Mpc.npy", arr)
    params = {"IO_DIR": str(tmp_path), "DIM": dim, "HII_DIM": sw, "BOX_LEN": np.float32(L),
              "PIXEL_FACTOR": np.float32(2.0), "MASS_FACTOR": np.float32(8.0), "INITIAL_REDSHIFT": 300.0,
              "COSMO": cos.PLANCK13}
    out = prog.run(8.0, params=params, linear=False)
    saved = np.load(boxes / "updated_smoothed_deltax_z8.00_32_100Mpc.npy")
    assert np.array_equal(out, saved)
    fg = np.float32(cos.growth_factor(8.0, cos.PLANCK13))
    fg0 = np.float32(cos.growth_factor(300.0, cos.PLANCK13))
    ref = PO.move_mass(delta, *v, fg0, np.float32((fg - fg0) / np.float32(L)), 2.0, 8.0)
    assert np.array_equal(out, ref)
    # the velocity boxes at z = 8 (perturb_field.py:110-125)
    rate = np.float32(cos.growth_rate(8.0, cos.PLANCK13))
    R = float(np.float32(np.float32(0.620350491) * np.float32(L) / np.float32(sw)))
    vref = PO.velocities(delta, sw, L, R, rate, 2.0)
    for c in "xyz":
        got = np.load(boxes / f"updated_v{c}overddot_32_100Mpc.npy")
        assert got.dtype == np.float32 and got.shape == (sw,) * 3
        assert _rel(got, vref["v" + c]) < 2e-5, c
    np.save(boxes / "smoothed_deltax_z0.00_32_100Mpc.npy", delta[:32, :32, :32].copy())
    lin = prog.run(8.0, params=params, linear=True)
    assert np.array_equal(lin, PO.evolve_linear(delta[:32, :32, :32], fg))
