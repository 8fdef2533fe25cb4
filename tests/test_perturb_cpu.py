"""CPU checks of the density-evolution oracle and of the drop-in program's host logic."""
import numpy as np
import pytest

from conftest import module
from oracle import pf_oracle as PO


def _fields(dim, sw, seed, vscale):
    rng = np.random.default_rng(seed)
    delta = rng.standard_normal((dim,) * 3).astype(np.float32) * np.float32(2.0)
    v = [rng.standard_normal((sw,) * 3).astype(np.float32) * np.float32(vscale) for _ in range(3)]
    return delta, v


def test_zero_displacement_is_the_block_mean():
    dim, sw, g0 = 32, 8, 0.01
    delta, _ = _fields(dim, sw, 0, 1.0)
    z = np.zeros((sw,) * 3, np.float32)
    out = PO.move_mass(delta, z, z, z, g0, 0.0, dim / sw, (dim / sw) ** 3)
    mass = (np.float32(1) + (np.float32(g0) * delta).astype(np.float32)).astype(np.float64)
    blocks = mass.reshape(sw, 4, sw, 4, sw, 4).mean(axis=(1, 3, 5)) - 1.0
    assert np.abs(out - blocks).max() < 2e-7


def test_mass_is_conserved_exactly():
    dim, sw = 32, 16
    delta, v = _fields(dim, sw, 1, 40.0)
    out, sums = PO.move_mass(delta, *v, 0.02, 0.01, dim / sw, (dim / sw) ** 3, return_sums=True)
    mass = (np.float32(1) + (np.float32(0.02) * delta).astype(np.float32)).astype(np.float64)
    q = np.rint(mass * 2.0 ** 32).astype(np.int64)
    assert int(sums.sum()) == int(q.sum())
    assert out.dtype == np.float32 and out.shape == (sw,) * 3


def test_whole_cell_shift_rolls_the_grid():
    # displacement of exactly one HII cell along each axis in turn (1/16 is exact in float32)
    dim, sw = 64, 16
    delta, _ = _fields(dim, sw, 2, 1.0)
    z = np.zeros((sw,) * 3, np.float32)
    one = np.full((sw,) * 3, 1.0 / 16.0, np.float32)
    base = PO.move_mass(delta, z, z, z, 0.05, 1.0, 4.0, 64.0)
    for axis in range(3):
        v = [z, z, z]
        v[axis] = one
        shifted = PO.move_mass(delta, *v, 0.05, 1.0, 4.0, 64.0)
        assert np.array_equal(shifted, np.roll(base, 1, axis=axis)), axis


def test_wrap_across_several_box_lengths():
    # a displacement of 2.5 box lengths lands where 0.5 box lengths does
    dim, sw = 16, 8
    delta, _ = _fields(dim, sw, 3, 1.0)
    half = np.full((sw,) * 3, 0.5, np.float32)
    far = np.full((sw,) * 3, 2.5, np.float32)
    a = PO.move_mass(delta, half, half, half, 0.1, 1.0, 2.0, 8.0)
    b = PO.move_mass(delta, far, far, far, 0.1, 1.0, 2.0, 8.0)
    assert np.array_equal(a, b)


def test_axis_tables_follow_float32_division():
    pos, hidx = PO.axis_tables(100, 64, np.float32(100) / np.float32(64))
    assert pos.dtype == np.float32 and pos[0] == np.float32(0.005)
    assert hidx.max() == 63 and (np.diff(hidx) >= 0).all()
    with pytest.raises(ValueError):
        PO.axis_tables(100, 32, 1.0)


def test_linear_evolution_and_file_names():
    pf = module("Programs.perturb_field")
    d = np.arange(8, dtype=np.float32).reshape(2, 2, 2)
    assert np.array_equal(PO.evolve_linear(d, 0.25), d * np.float32(0.25))
    p = {"HII_DIM": 128, "BOX_LEN": 300.0}
    assert pf.output_name(12.0, p) == "updated_smoothed_deltax_z12.00_128_300Mpc"
    g = pf.growth(0.0, module("Programs._common").params())
    assert g == np.float32(1.0)


def test_growth_rate_limits():
    cos = module("cosmology")
    P = cos.PLANCK13
    # matter domination: D grows as a, so (dD/dt) / D = H(z)
    assert abs(cos.growth_rate(50.0, P) / cos.hubble(50.0, P) - 1.0) < 1e-4
    # today: f = dlnD/dlna near Om^0.55 (Linder 2005), within the Carroll-Press-Turner fit
    f0 = cos.growth_rate(0.0, P) / cos.hubble(0.0, P)
    assert abs(f0 / P.omega_M_0 ** 0.55 - 1.0) < 0.04
    # H0 = 100 h km/s/Mpc in 1/s
    assert abs(cos.hubble(0.0, P) / (P.h * 3.2407792894e-18) - 1.0) < 1e-9


def test_velocity_divergence_is_minus_rate_times_smoothed_density():
    # with nearest-cell subsampling at pixel factor 1, div v = -(dD/dt / D) delta_smoothed on every
    # non-zero mode except the Nyquist planes, whose derivative the velocity boxes drop
    from oracle import es_oracle
    n, L, R, rate = 32, 64.0, 1.5, 2.0
    rng = np.random.default_rng(4)
    d = rng.standard_normal((n,) * 3)
    v = PO.velocities(d, n, L, R, rate, 1.0)
    dk = float(np.float32(2 * np.pi / L))
    m = np.fft.fftfreq(n, d=1.0 / n)
    mz = np.arange(n // 2 + 1)
    k2 = (m[:, None, None] ** 2 + m[None, :, None] ** 2 + mz[None, None, :] ** 2).astype(np.int64)
    div = (1j * dk * m[:, None, None] * np.fft.rfftn(v["vx"]) + 1j * dk * m[None, :, None] * np.fft.rfftn(v["vy"])
           + 1j * dk * mz[None, None, :] * np.fft.rfftn(v["vz"]))
    smooth = np.fft.rfftn(d) * es_oracle.window(k2, dk, R, 0, False)
    keep = (np.abs(m[:, None, None]) < n // 2) & (np.abs(m[None, :, None]) < n // 2) & (mz[None, None, :] < n // 2)
    keep = np.broadcast_to(keep, div.shape) & (k2 > 0)          # the mean has no velocity
    err = np.abs(div + float(np.float32(rate)) * smooth)[keep].max()
    assert err < 1e-9 * np.abs(smooth).max()
    assert all(x.shape == (n,) * 3 for x in v.values())


def test_velocity_file_names():
    pf = module("Programs.perturb_field")
    p = {"HII_DIM": 128, "BOX_LEN": 300.0}
    assert pf.velocity_name("x", p) == "updated_vxoverddot_128_300Mpc"
