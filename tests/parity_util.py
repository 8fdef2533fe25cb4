"""Parity bars shared by the GPU tests (imported by the test modules; collects no tests).

Ionisation flags agree except in cells within 1e-5 of the threshold (the union of spheres around
such centres in sphere mode); mean x_HI and P(k) agree to 1e-4 relative; partial ionisations
(final radius) agree to 2e-4 absolute (float32 transforms against float64).
"""
import numpy as np

FLAG_TOL = 1e-5
MEAN_RTOL = 1e-4
PK_RTOL = 1e-4
PARTIAL_ATOL = 2e-4


def compare_ionized(ion_gpu, ref, label=""):
    """Every cell outside the oracle's exemption band must match the oracle's ionised fraction.

    Loop radii decide flags (a flip there changes the cell from 1 to a partial value, far
    beyond the tolerance); the final radius is continuous at the threshold (zeta f -> 1 from
    below meets the flagged value 1), so it needs no exemption.
    """
    ion_o = ref["ionized"]
    ex = ref["exempt"]
    diff = np.abs(ion_gpu - ion_o)
    bad = (diff > PARTIAL_ATOL) & ~ex
    assert bad.sum() == 0, (f"{label}: {int(bad.sum())} cells differ by more than {PARTIAL_ATOL} outside "
                            f"the {int(ex.sum())} exempt cells (max {diff[~ex].max():.3g})")
    loop_flags = ref["flags"]
    assert np.all(ion_gpu[loop_flags & ~ex] == 1.0), f"{label}: oracle-flagged cells not ionised"
    xg, xo = 1.0 - ion_gpu.mean(), 1.0 - ion_o.mean()
    assert abs(xg - xo) <= MEAN_RTOL * abs(xo) + 1e-7, f"{label}: mean x_HI {xg} vs {xo}"


def compare_pk(pk_gpu, oracle_pk, label=""):
    """P(k) rows (ps_ave, k_ave, count) against the oracle's (K, k_ave, ps_ave, count)."""
    _K, k_ave, ps_ave, cnt = oracle_pk
    assert np.array_equal(pk_gpu[2], cnt.astype(np.float32)), f"{label}: mode counts differ"
    nz = cnt > 0
    assert np.allclose(pk_gpu[1][nz], k_ave[nz], rtol=1e-5), f"{label}: k_ave differs"
    rel = np.abs(pk_gpu[0][nz] - ps_ave[nz]) / np.abs(ps_ave[nz])
    assert rel.max() <= PK_RTOL, f"{label}: P(k) relative error {rel.max():.3g}"
