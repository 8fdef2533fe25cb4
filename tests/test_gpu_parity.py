"""Parity of the CUDA engine (through the C ABI) with the FP64 oracle on seeded inputs.

Bars (from the engine's contract): ionisation flags agree except in cells within 1e-5 of the
threshold; mean x_HI and P(k) agree to 1e-4 relative; partial ionisations agree to 2e-4
absolute (float32 transforms against float64).
"""
import os

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import es_oracle as O  # noqa: E402
from parity_util import FLAG_TOL, MEAN_RTOL, PARTIAL_ATOL, PK_RTOL, compare_ionized, compare_pk  # noqa: E402,F401

cos = module("cosmology")
sch = module("schedule")
grf = module("grf")


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return module("engine")


def _plan(eng, n, L, max_radii=64):
    return eng.ExcursionSetPlan(n, L, max_radii=max_radii)


def _setup(n, L, z, **kw):
    base = dict(zeta=30.0, t_vir_min=1e4, R_max=15.0, cosmo=cos.BASELINE_COSMO)
    base.update(kw)
    return sch.ionize_setup(n, L, z, **base)


_compare_ionized = compare_ionized


@pytest.mark.parametrize("n", [16, 32, 48, 64, 96, 128, 160])
def test_fft_matches_numpy(eng, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n, n)).astype(np.float32)
    with _plan(eng, n, 100.0) as p:
        X = p.fft_r2c(torch.from_numpy(x).cuda()).cpu().numpy()
        ref = np.fft.rfftn(x.astype(np.float64))
        err = np.abs(X - ref).max() / np.abs(ref).max()
        assert err < 2e-6, f"forward rel err {err}"
        y = p.fft_c2r(torch.from_numpy(ref.astype(np.complex64)).cuda()).cpu().numpy() / n ** 3
        err2 = np.abs(y - x).max() / np.abs(x).max()
        assert err2 < 2e-6, f"inverse rel err {err2}"


@pytest.mark.parametrize("n", [256, 512, 1024])
def test_fft_roundtrip_full_size(eng, n):
    # size-independent property at the benchmark sizes: c2r(r2c(x)) / n^3 == x, Parseval,
    # and agreement with torch.fft (cuFFT, used here only as a checker)
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn((n, n, n), device="cuda", generator=g, dtype=torch.float32)
    with _plan(eng, n, 300.0) as p:
        X = p.fft_r2c(x)
        ref = torch.fft.rfftn(x)
        rel = ((X - ref).abs().max() / ref.abs().max()).item()
        assert rel < 3e-6, rel
        y = p.fft_c2r(X) / n ** 3
        assert ((y - x).abs().max() / x.abs().max()).item() < 3e-6
        del X, ref, y
        torch.cuda.empty_cache()


CASES = [
    # (n, L, z, kwargs)
    (16, 24.0, 8.0, dict(R_max=6.0)),
    (32, 48.0, 8.0, dict()),
    (64, 100.0, 8.0, dict()),                                   # the CPU-runnable 64^3 case
    (64, 100.0, 8.0, dict(filter_type=1)),
    (64, 100.0, 8.0, dict(filter_type=2)),
    (64, 100.0, 8.0, dict(ref_compat=True)),
    (64, 100.0, 8.0, dict(ref_compat=True, filter_type=1)),
    (64, 100.0, 10.0, dict(linear=True)),
    (48, 72.0, 7.0, dict(zeta=50.0, R_max=20.0)),
    (96, 144.0, 9.0, dict(zeta=20.0, R_max=8.0, t_vir_min=3e4)),
    (160, 240.0, 6.5, dict(zeta=60.0, R_max=40.0)),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{i}" for i, c in enumerate(CASES)])
def test_ionize_matches_oracle(eng, case):
    n, L, z, kw = case
    d = grf.density_box(n, L, seed=n + 3, z=z)
    st = _setup(n, L, z, **kw)
    ref = O.conv_bubbles(d, st, tol=FLAG_TOL)
    with _plan(eng, n, L) as p:
        out, nf = p.run(torch.from_numpy(d).cuda(), st, output="ionized")
        ion32 = out.cpu().numpy()
        ion = ion32.astype(np.float64)
        xh, nfv = p.run(torch.from_numpy(d).cuda(), st, output="xH")
        assert np.array_equal(xh.cpu().numpy(), np.float32(1.0) - ion32)
        assert abs(nfv.item() - (1.0 - ion.mean())) < 1e-5
    _compare_ionized(ion, ref, f"n={n} {kw}")


@pytest.mark.parametrize("ref_compat", [False, True])
def test_sphere_painting_matches_oracle(eng, ref_compat):
    n, L, z = 32, 48.0, 8.0
    d = grf.density_box(n, L, seed=11, z=z)
    st = _setup(n, L, z, update=1, ref_compat=ref_compat, R_max=10.0)
    ref = O.conv_bubbles(d, st, tol=FLAG_TOL)
    with _plan(eng, n, L) as p:
        out, _ = p.run(torch.from_numpy(d).cuda(), st, output="ionized")
    _compare_ionized(out.cpu().numpy().astype(np.float64), ref, f"sphere ref_compat={ref_compat}")


@pytest.mark.parametrize("n,L", [(32, 48.0), (48, 72.0), (96, 144.0), (256, 300.0)])
def test_tile_variants_agree(eng, n, L):
    # every tile-shape candidate of the autotuner (TMA and synchronous passes) runs the same
    # transforms; they differ only in where the compiler contracts the filter multiply into FMAs
    # and, with capped row-pass grids, in the order of the grid-wide erfc sum
    at = module("autotune")
    z = 8.0
    d = torch.from_numpy(grf.density_box(n, L, seed=1, z=z)).cuda()
    st = _setup(n, L, z, R_max=min(15.0, 0.2 * L))
    c = cos.brightness_temperature_factor(z, cos.BASELINE_COSMO)
    edges = sch.pk_edges(n, L, 20)
    outs = {}
    # plus the overlapped-radius schedules on the first tile configuration
    configs = list(at.CANDIDATES) + [at.with_overlap(at.CANDIDATES[0], ov) for ov in at.OVERLAP[1:]]
    with _plan(eng, n, L) as p:
        for cfg in configs:
            at.apply(p, cfg)
            xh, nf = p.run(d, st)
            dT, ave = p.delta_T(xh, d, c)
            pk = p.power_spectrum(dT, ave, edges)
            X = p.fft_r2c(d)
            outs[cfg] = (xh.clone(), nf.item(), pk.clone(), X.clone())
        p.check()
    ref = outs[at.CANDIDATES[0]]
    for cfg, (xh, nf, pk, X) in outs.items():
        diff = (xh - ref[0]).abs()
        assert (diff > PARTIAL_ATOL).float().mean().item() <= 1e-5, cfg
        assert abs(nf - ref[1]) <= 1e-6, cfg
        assert torch.equal(pk[2], ref[2][2]), cfg
        nz = ref[2][2] > 0
        assert torch.allclose(pk[0][nz], ref[2][0][nz], rtol=1e-5), cfg
        assert ((X - ref[3]).abs().max() / ref[3].abs().max()).item() < 1e-6, cfg


def test_sum_erfc_against_library_and_float64(eng):
    # the per-radius fcoll sum uses Numerical Recipes' erfcc; check it against CUDA's erfcf and
    # against float64 scipy over the arguments the engine meets (and well beyond)
    import ctypes as C
    from scipy.special import erfc
    _lib = module("_lib")
    lib = _lib.load()
    x = torch.linspace(-6.0, 10.0, 400001, device="cuda")
    fast, ref = torch.empty_like(x), torch.empty_like(x)
    rc = lib.es_selftest_erfc(C.c_void_p(x.data_ptr()), C.c_void_p(fast.data_ptr()), C.c_void_p(ref.data_ptr()),
                              x.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("es_selftest_erfc", rc, lib)
    xd = x.cpu().numpy().astype(np.float64)
    exact = erfc(xd)
    keep = exact > 1e-30
    rel_fast = np.abs(fast.cpu().numpy()[keep] - exact[keep]) / exact[keep]
    rel_lib = np.abs(ref.cpu().numpy()[keep] - exact[keep]) / exact[keep]
    # the cells that carry the sum have |x| < 3 (erfc > 2e-5); beyond, a few 1e-6 do not matter
    core = np.abs(xd[keep]) < 3.0
    assert rel_fast[core].max() < 2e-6, rel_fast[core].max()
    assert rel_fast.max() < 2e-5, rel_fast.max()
    assert rel_lib.max() < 1e-6
    # what the engine uses it for: the mean over cells, here weighted like a smoothed density
    # field's x = (delta_c - delta_R) / denom, must agree to well below the 1e-5 flag tolerance
    w = np.exp(-0.5 * ((xd - 1.5) / 1.0) ** 2)
    mean_fast = np.sum(w * fast.cpu().numpy()) / np.sum(w)
    mean_exact = np.sum(w * exact) / np.sum(w)
    assert abs(mean_fast / mean_exact - 1) < 2e-7
    # no bias: the mean signed error over a band of typical arguments stays tiny
    band = (xd > -1) & (xd < 4)
    signed = (fast.cpu().numpy()[band] - exact[band]) / exact[band]
    assert abs(signed.mean()) < 1e-7


def test_ionize_is_deterministic(eng):
    n, L, z = 64, 100.0, 8.0
    d = torch.from_numpy(grf.density_box(n, L, seed=0, z=z)).cuda()
    st = _setup(n, L, z)
    with _plan(eng, n, L) as p:
        a, na = p.run(d, st)
        a = a.clone(); na = na.clone()
        b, nb = p.run(d, st)
    assert torch.equal(a, b) and torch.equal(na, nb)


def test_uniform_density_hand_derived(eng):
    # a uniform box keeps delta_R constant for every R (W(0) = 1); after the mean
    # normalisation every cell has f = fc_mean_ps, so the box is fully ionised iff
    # zeta * fc_mean_ps >= 1, otherwise x_HI = 1 - zeta * fc_mean_ps everywhere
    n, L, z = 32, 48.0, 8.0
    for zeta, expect_full in [(40.0, True), (20.0, False)]:
        st = _setup(n, L, z, zeta=zeta)
        fc = float(st.fc_mean_ps)
        assert (zeta * fc >= 1.0) == expect_full
        d = torch.full((n, n, n), 0.3, dtype=torch.float32, device="cuda")
        with _plan(eng, n, L) as p:
            xh, nf = p.run(d, st)
        want = 0.0 if expect_full else 1.0 - zeta * fc
        assert torch.allclose(xh, torch.full_like(xh, want), atol=2e-5), (xh.min().item(), xh.max().item(), want)


def test_delta_T_and_power_spectrum_match_oracle(eng):
    n, L, z = 64, 100.0, 8.0
    d = grf.density_box(n, L, seed=0, z=z)
    st = _setup(n, L, z)
    c = cos.brightness_temperature_factor(z, cos.BASELINE_COSMO)
    edges = sch.pk_edges(n, L, 20)
    with _plan(eng, n, L) as p:
        dd = torch.from_numpy(d).cuda()
        xh, _ = p.run(dd, st)
        dT, ave = p.delta_T(xh, dd, c)
        pk = p.power_spectrum(dT, ave, edges).cpu().numpy()
        xh_h = xh.cpu().numpy()
        dT_h = dT.cpu().numpy()
        ave_h = ave.item()
    dT_o, ave_o = O.delta_T(xh_h, d, c)
    assert abs(ave_h - ave_o) <= 1e-5 * abs(ave_o)
    assert np.abs(dT_h - dT_o).max() <= 1e-5 * np.abs(dT_o).max()
    K, k_ave, ps_ave, cnt = O.power_spectrum(dT_o, ave_o, L, edges)
    assert np.array_equal(pk[2], cnt.astype(np.float32)), (pk[2], cnt)
    nz = cnt > 0
    assert np.allclose(pk[1][nz], k_ave[nz], rtol=1e-5)
    rel = np.abs(pk[0][nz] - ps_ave[nz]) / np.abs(ps_ave[nz])
    assert rel.max() <= PK_RTOL, rel


def test_power_spectrum_dimensional_and_ragged_bins(eng):
    n, L = 48, 75.0
    rng = np.random.default_rng(5)
    dT = (20.0 + rng.standard_normal((n, n, n))).astype(np.float32)
    for nbins, dim in [(1, False), (7, True), (100, False), (128, True)]:
        edges = sch.pk_edges(n, L, nbins)
        with _plan(eng, n, L) as p:
            t = torch.from_numpy(dT).cuda()
            ave = torch.tensor([float(dT.astype(np.float64).mean())], dtype=torch.float32, device="cuda")
            pk = p.power_spectrum(t, ave, edges, dimensional=dim).cpu().numpy()
        _, k_ave, ps_ave, cnt = O.power_spectrum(dT, float(ave.item()), L, edges, dimensional=dim)
        assert np.array_equal(pk[2], cnt.astype(np.float32))
        nz = cnt > 0
        assert np.allclose(pk[0][nz], ps_ave[nz], rtol=PK_RTOL, atol=0)


@pytest.mark.skipif(os.environ.get("ES_SKIP_FULL") == "1", reason="full-size parity disabled")
def test_full_size_256_box_matches_oracle(eng):
    # one box of the 256^3 sweep, against the oracle run with multithreaded scipy.fft: ionisation,
    # then delta_T and the 20-bin P(k) of the engine's x_HI against the oracle's on the same x_HI
    # (delta_T.py:73-98)
    b = grf.sweep_256()[5]
    d = grf.density_box(b.n, b.box_len, b.seed, b.z)
    st = _setup(b.n, b.box_len, b.z, zeta=b.zeta, R_max=b.R_max, t_vir_min=b.t_vir_min)
    assert st.n_radii == 32
    ref = O.conv_bubbles(d, st, tol=FLAG_TOL, backend="scipy", workers=os.cpu_count())
    c = cos.brightness_temperature_factor(b.z, cos.BASELINE_COSMO)
    edges = sch.pk_edges(b.n, b.box_len, 20)
    with _plan(eng, b.n, b.box_len) as p:
        dd = torch.from_numpy(d).cuda()
        out, _ = p.run(dd, st, output="ionized")
        ion = out.cpu().numpy().astype(np.float64)
        xh, _ = p.run(dd, st)
        dT, ave = p.delta_T(xh, dd, c)
        pk = p.power_spectrum(dT, ave, edges).cpu().numpy()
        xh_h, dT_h, ave_h = xh.cpu().numpy(), dT.cpu().numpy(), ave.item()
    _compare_ionized(ion, ref, "256^3")
    dT_o, ave_o = O.delta_T(xh_h, d, c)
    assert abs(ave_h - ave_o) <= 1e-5 * abs(ave_o)
    assert np.abs(dT_h - dT_o).max() <= 1e-5 * np.abs(dT_o).max()
    compare_pk(pk, O.power_spectrum(dT_o, ave_o, b.box_len, edges, backend="scipy", workers=os.cpu_count()), "256^3")


@pytest.mark.parametrize("update", [0, 1])
def test_overlapped_radii_match_serial_schedule(eng, update):
    # the column passes of radius r + 1 on the plan's own stream beside the row pass (and, in
    # sphere mode, the painting) of radius r: the same flags and x_HI as the serial schedule, and
    # the oracle's, for centre and sphere updates; capped grids only reorder the erfc sum
    _lib = module("_lib")
    n, L, z = 96, 144.0, 8.0
    d = grf.density_box(n, L, seed=21, z=z)
    st = _setup(n, L, z, update=update, R_max=12.0)
    dd = torch.from_numpy(d).cuda()
    with _plan(eng, n, L) as p:
        serial, _ = p.run(dd, st, output="ionized")
        serial = serial.clone()
        for ov in ((1, 0, 0), (1, 1, 2), (1, 2, 1)):
            for opt, v in zip((_lib.OPT_OVERLAP, _lib.OPT_ROW_CTAS, _lib.OPT_COL_CTAS), ov):
                p.set_option(opt, v)
            out, _ = p.run(dd, st, output="ionized")
            if ov[1] == 0:
                assert torch.equal(out, serial), ov
            else:
                assert (out != serial).float().mean().item() <= 1e-4, ov
        p.check()
    ref = O.conv_bubbles(d, st, tol=FLAG_TOL)
    _compare_ionized(out.cpu().numpy().astype(np.float64), ref, f"overlap update={update}")
