"""Parity pinned to the reference's own kernels (three-way, on the same seeded inputs).

The reference's Programs/find_bubbles.cu, compiled from its own source after its own templating
(oracle/build_ref.py), is driven by a harness that follows conv_bubbles
(find_HII_bubbles.py:83-192) line by line with torch.fft in place of pyfft
(oracle/ref_harness.py).  In ``ref_compat`` mode the engine reproduces the reference's kernel
semantics (the HII_filter switch fall-through, the sphere radius in Mpc used as cells and the
clamped painting), so three results must agree under the same bars:

* the CUDA engine against the FP64 oracle,
* the reference's kernels against the FP64 oracle,
* the CUDA engine against the reference's kernels (cells outside the oracle's exemption band).

The reference's kernels reach the GPU machine as the staged copy under oracle/_ref (made where a
checkout of the reference exists); without it the tests skip and say so.
"""
import os

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import build_ref  # noqa: E402
from oracle import es_oracle as O  # noqa: E402
from parity_util import FLAG_TOL, MEAN_RTOL, PARTIAL_ATOL, compare_ionized  # noqa: E402

cos = module("cosmology")
sch = module("schedule")
grf = module("grf")

CASES = [
    # (n, L, z, seed, kwargs) -- all with ref_compat=True
    (64, 100.0, 8.0, 0, dict()),                                    # the 64^3 configuration, filter 0
    (64, 100.0, 8.0, 0, dict(filter_type=1)),
    (64, 100.0, 8.0, 0, dict(filter_type=2)),
    (64, 100.0, 10.0, 4, dict(linear=True)),                        # LE=True: no rescale, no normalisation
    (64, 100.0, 8.0, 5, dict(update=1, R_max=8.0)),                 # sphere painting, R (Mpc) as cells
    (128, 200.0, 7.0, 6, dict(zeta=50.0, R_max=20.0)),
    (128, 192.0, 9.0, 7, dict(filter_type=1, zeta=20.0)),
]


@pytest.fixture(scope="module")
def eng():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build_ref.stage()
    if not build_ref.available():
        pytest.skip("the reference's find_bubbles.cu is not staged under oracle/_ref (no reference checkout "
                    "where the repository was prepared)")
    return module("engine")


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{i}" for i, c in enumerate(CASES)])
def test_engine_oracle_and_reference_kernels_agree(eng, case):
    from oracle.ref_harness import conv_bubbles_ref
    n, L, z, seed, kw = case
    d = grf.density_box(n, L, seed=seed, z=z)
    args = dict(zeta=30.0, t_vir_min=1e4, R_max=15.0, cosmo=cos.BASELINE_COSMO, ref_compat=True)
    args.update(kw)
    st = sch.ionize_setup(n, L, z, **args)
    ref = O.conv_bubbles(d, st, tol=FLAG_TOL, backend="scipy", workers=os.cpu_count() or 1)
    ion_ref, sums = conv_bubbles_ref(d, st)
    with eng.ExcursionSetPlan(n, L) as p:
        out, _ = p.run(torch.from_numpy(d).cuda(), st, output="ionized")
        ion_eng = out.cpu().numpy()
    label = f"n={n} {kw}"
    # the reference's kernels against the FP64 restatement
    compare_ionized(ion_ref.astype(np.float64), ref, label + " reference kernels vs oracle")
    # the engine against the FP64 restatement
    compare_ionized(ion_eng.astype(np.float64), ref, label + " engine vs oracle")
    # the engine against the reference's kernels, outside the band where float32 and float64 may
    # legitimately decide differently
    ex = ref["exempt"]
    diff = np.abs(ion_eng.astype(np.float64) - ion_ref.astype(np.float64))
    bad = (diff > PARTIAL_ATOL) & ~ex
    assert bad.sum() == 0, f"{label}: engine and reference kernels differ in {int(bad.sum())} cells"
    xe, xr = 1.0 - ion_eng.mean(dtype=np.float64), 1.0 - ion_ref.mean(dtype=np.float64)
    assert abs(xe - xr) <= MEAN_RTOL * abs(xr) + 1e-7, (xe, xr)
    # per-radius <fcoll> of the reference's kernels (float32 erfcf, float32 sum) against float64
    means = np.asarray(sums, dtype=np.float64) / float(n) ** 3
    loop = [i for i, s in enumerate(st.steps)]
    rel = np.abs(means[loop] - ref["means"][loop]) / np.abs(ref["means"][loop])
    assert rel.max() < 1e-4, (label, rel.max())
