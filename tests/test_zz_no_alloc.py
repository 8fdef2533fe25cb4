"""The allocation-free delta_T entry point against the plan-based one, through the C ABI.

es_delta_T_noalloc exists for callers that cannot call cudaMalloc (code running inside another
runtime's memory pool, hosts that only hand over device pointers, embedders that forbid
allocation after start-up): its scratch is a static device array.  This file is collected last
so that a failure here cannot hide the result of any other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-6      # same kernel and grid as es_delta_T: the results are expected to be identical


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("_lib").load()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("n", [64, 256])     # 256^3: every CTA's grid-stride loop runs many times
def test_noalloc_delta_T_matches_plan_entry_point_twice(lib, n):
    _lib = module("_lib")
    eng = module("engine")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    with eng.ExcursionSetPlan(n, 1.5 * n) as plan:
        for call, seed in enumerate((1, 2)):           # two calls in a row, different inputs
            g = torch.Generator(device="cuda").manual_seed(seed)
            xH = torch.rand((n, n, n), device="cuda", generator=g)
            delta = torch.randn((n, n, n), device="cuda", generator=g) * 0.5
            c = 23.5 + call
            dT_ref = torch.empty_like(xH)
            ave_ref = torch.empty(1, device="cuda")
            rc = lib.es_delta_T(plan.handle, _ptr(xH), _ptr(delta), C.c_float(c), _ptr(dT_ref), _ptr(ave_ref), stream)
            _lib.check("es_delta_T", rc, lib)
            dT = torch.full_like(xH, float("nan"))
            ave = torch.full((1,), float("nan"), device="cuda")
            rc = lib.es_delta_T_noalloc(n, _ptr(xH), _ptr(delta), C.c_float(c), _ptr(dT), _ptr(ave), stream)
            _lib.check("es_delta_T_noalloc", rc, lib)
            torch.cuda.synchronize()
            assert torch.allclose(dT, dT_ref, rtol=RTOL, atol=0.0)
            assert abs(ave.item() - ave_ref.item()) <= RTOL * abs(ave_ref.item())
            want = (c * xH.double() * (1.0 + delta.double())).mean().item()
            assert abs(ave.item() - want) <= 1e-5 * abs(want)


def test_noalloc_rejects_sizes_beyond_its_maximum(lib):
    _lib = module("_lib")
    x = torch.zeros(8, device="cuda")
    for n in (2048, 63, 0):
        rc = lib.es_delta_T_noalloc(n, _ptr(x), _ptr(x), C.c_float(1.0), _ptr(x), _ptr(x), None)
        assert rc == -1
        assert "HII_DIM" in _lib.last_error(lib)
    assert np.isfinite(x.cpu().numpy()).all()
