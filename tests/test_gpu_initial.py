"""Initial conditions on the GPU against their CPU restatement, statistics, and the
initialize -> perturb_field -> find_HII_bubbles chain (GPU)."""
import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import ic_oracle as IO  # noqa: E402
from oracle import pf_oracle as PO  # noqa: E402

cos = module("cosmology")


@pytest.fixture(scope="module")
def ini():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("initial")


def _normals(n, seed):
    rng = np.random.default_rng(seed)
    shape = (n, n, n // 2 + 1)
    return rng.standard_normal(shape).astype(np.float32), rng.standard_normal(shape).astype(np.float32)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_spectrum_is_bit_exact(ini):
    n, L = 64, 100.0
    nre, nim = _normals(n, 0)
    with ini.InitialConditions(n, 32, L) as ic:
        H = ic.spectrum(torch.from_numpy(nre).cuda(), torch.from_numpy(nim).cuda()).cpu().numpy()
        K, P = ic.K.cpu().numpy(), ic.P.cpu().numpy()
    ref = IO.spectrum(n, L, nre, nim, K, P)
    assert np.array_equal(H.real, ref.real.astype(np.float32)) and np.array_equal(H.imag, ref.imag.astype(np.float32))


@pytest.mark.parametrize("ref_compat", [False, True])
def test_boxes_match_float64_restatement(ini, ref_compat):
    n, sw, L = 64, 32, 100.0
    nre, nim = _normals(n, 1)
    with ini.InitialConditions(n, sw, L) as ic:
        out = ic.generate(normals=(torch.from_numpy(nre).cuda(), torch.from_numpy(nim).cuda()), ref_compat=ref_compat)
        H = out["spectrum"].cpu().numpy()
        R = ic.smooth_R
    ref = IO.boxes(H, L, sw, R, 0, ref_compat)
    for name in ("deltax", "smoothed", "vx", "vy", "vz"):
        assert out[name].shape == ref[name].shape, name
        assert _rel(out[name].cpu().numpy(), ref[name]) < 2e-5, name


def test_density_power_spectrum_is_the_input_one(ini):
    n, L = 128, 200.0
    with ini.InitialConditions(n, 64, L) as ic:
        d = ic.generate(seed=3)["deltax"].cpu().numpy().astype(np.float64)
    F = np.fft.rfftn(d)
    pk = np.abs(F) ** 2 * L ** 3 / n ** 6
    dk = 2 * np.pi / L
    m = np.fft.fftfreq(n, d=1.0 / n)
    kk = dk * np.sqrt(m[:, None, None] ** 2 + m[None, :, None] ** 2 + np.arange(n // 2 + 1)[None, None, :] ** 2)
    edges = np.logspace(np.log10(2 * dk), np.log10(dk * n / 4), 9)
    ratios = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        sel = (kk >= lo) & (kk < hi)
        if sel.sum() < 200:
            continue
        ratios.append(pk[sel].mean() / cos.power_spectrum_z0(kk[sel], cos.PLANCK13).mean())
    ratios = np.array(ratios)
    assert len(ratios) >= 5
    assert np.all(np.abs(ratios - 1) < 0.2), ratios
    assert abs(ratios.mean() - 1) < 0.06, ratios


def test_displacement_divergence_is_minus_the_smoothed_density(ini):
    # with HII_DIM = DIM the subsample is the identity: div(psi) = -delta_smoothed mode by mode
    n, L = 64, 100.0
    with ini.InitialConditions(n, n, L) as ic:
        out = ic.generate(seed=5)
    dk = 2 * np.pi / L
    m = np.fft.fftfreq(n, d=1.0 / n)
    k = (m[:, None, None] * dk, m[None, :, None] * dk, np.arange(n // 2 + 1)[None, None, :] * dk)
    div = sum(1j * k[c] * np.fft.rfftn(out[v].cpu().numpy().astype(np.float64)) for c, v in enumerate(("vx", "vy", "vz")))
    S = np.fft.rfftn(out["smoothed"].cpu().numpy().astype(np.float64))
    # modes off every Nyquist index (where an odd derivative has no real value) and off k = 0
    inner = (np.abs(m)[:, None, None] < n // 2) & (np.abs(m)[None, :, None] < n // 2) & \
            (np.arange(n // 2 + 1)[None, None, :] < n // 2)
    inner[0, 0, 0] = False
    assert np.linalg.norm((div + S)[inner]) / np.linalg.norm(S[inner]) < 1e-4


def test_initialize_perturb_ionize_chain(ini, tmp_path):
    init = module("Programs.initialize")
    pert = module("Programs.perturb_field")
    fhb = module("Programs.find_HII_bubbles")
    params = {"IO_DIR": str(tmp_path), "DIM": 64, "HII_DIM": 32, "BOX_LEN": np.float32(64.0),
              "PIXEL_FACTOR": np.float32(2.0), "MASS_FACTOR": np.float32(8.0), "INITIAL_REDSHIFT": 300.0,
              "COSMO": cos.PLANCK13}
    boxes = init.init(params=params, seed=7)
    assert set(boxes) == {"deltax_z0.00_64_64Mpc", "smoothed_deltax_z0.00_32_64Mpc", "vxoverddot_32_64Mpc",
                          "vyoverddot_32_64Mpc", "vzoverddot_32_64Mpc"}
    updated = pert.run(8.0, params=params, linear=False)
    fg = np.float32(cos.growth_factor(8.0, cos.PLANCK13))
    fg0 = np.float32(cos.growth_factor(300.0, cos.PLANCK13))
    ref = PO.move_mass(boxes["deltax_z0.00_64_64Mpc"], boxes["vxoverddot_32_64Mpc"], boxes["vyoverddot_32_64Mpc"],
                       boxes["vzoverddot_32_64Mpc"], fg0, np.float32((fg - fg0) / np.float32(64.0)), 2.0, 8.0)
    assert np.array_equal(updated, ref)
    pd = {"BoxSize": 64.0, "HIIdim": 32, "dim": 32, "z": 8.0}
    ion = fhb.conv_bubbles(updated, pd, Z=8.0, fil=0, params={"ZETA": 30.0, "R_BUBBLE_MAX": 10.0})
    assert np.isfinite(ion).all() and ion.min() >= 0.0 and ion.max() <= 1.0
