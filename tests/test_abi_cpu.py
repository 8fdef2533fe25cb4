"""CPU checks of the C ABI library and the host layer (no GPU calls)."""
import ctypes as C
import importlib
import re
from pathlib import Path

import pytest

from conftest import ROOT, module

HEADER = Path(ROOT) / "include" / "es_engine.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|size_t|const char\*)\s+((?:es|sg|pf|ic)_\w+)\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build = importlib.import_module("21cmpy_gb300._build")
    path = build.build()
    return C.CDLL(str(path))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/es_engine.h but not exported"


def test_binding_covers_the_header():
    _lib = module("_lib")
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_host_only_calls(lib):
    lib.es_supported_sizes.restype = C.c_int
    buf = (C.c_int * 16)()
    n = lib.es_supported_sizes(buf, 16)
    sizes = [buf[i] for i in range(n)]
    assert sizes == [16, 32, 48, 64, 96, 128, 160, 256, 512, 1024]
    lib.es_plan_workspace_bytes.restype = C.c_size_t
    lib.es_plan_workspace_bytes.argtypes = [C.c_int, C.c_int]
    assert lib.es_plan_workspace_bytes(100, 10) == 0          # unsupported size
    w = lib.es_plan_workspace_bytes(256, 40)
    assert 300e6 < w < 500e6
    # input spectrum, two intermediate spectra, two delta_R boxes, centre list, per-radius window
    # tables: 420 MB at 256^3 and 3.3 GB at 512^3 with room for 64 radii
    assert abs(lib.es_plan_workspace_bytes(256, 64) / 420e6 - 1) < 0.02
    assert abs(lib.es_plan_workspace_bytes(512, 64) / 3.3e9 - 1) < 0.02
    lib.es_version.restype = C.c_int
    assert lib.es_version() >= 1


def test_null_arguments_are_rejected_without_a_device(lib):
    _lib = module("_lib")
    L = _lib.load()
    assert L.es_plan_create(256, 300.0, 10, None) == -1
    assert "NULL" in _lib.last_error(L)
    h = C.c_void_p()
    assert L.es_plan_create(100, 300.0, 10, C.byref(h)) == -4        # no kernels for 100^3
    assert L.es_plan_create(64, -1.0, 10, C.byref(h)) == -1
    assert L.es_forward(None, None, None) == -1
    assert L.es_ionize(None, None, None, None, None) == -1


def test_engine_refuses_to_run_without_cuda():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    eng = module("engine")
    with pytest.raises(module("_lib").EngineUnavailable):
        eng.ExcursionSetPlan(64, 100.0)


def test_density_evolution_and_initial_condition_arguments_are_checked_without_a_device():
    _lib = module("_lib")
    L = _lib.load()
    h = C.c_void_p()
    assert L.pf_plan_create(64, 32, C.c_float(2.0), None) == -1
    assert L.pf_plan_create(32, 64, C.c_float(0.5), C.byref(h)) == -1        # HII_DIM above DIM
    assert L.pf_plan_create(64, 32, C.c_float(1.0), C.byref(h)) == -1        # indices leave the 32^3 grid
    buf = C.create_string_buffer(256)
    L.pf_last_error(buf, 256)
    assert b"leaves the 32^3 grid" in buf.value
    assert L.pf_move_mass(None, None, None, None, None, C.c_float(0), C.c_float(0), C.c_float(1), None, None) == -1
    assert L.pf_evolve_linear(-1, None, C.c_float(1), None, None) == -1
    assert L.pf_evolve_linear(0, None, C.c_float(1), None, None) == 0         # nothing to do
    assert L.ic_spectrum(1, C.c_float(100.0), None, None, None, None, 512, None, None) == -1
    assert L.ic_shape(64, C.c_float(100.0), None, 3, 0, C.c_float(1.0), 0, None, None) == -1
    assert L.ic_subsample(32, 64, C.c_float(0.5), C.c_float(1.0), None, None, None) == -1
    L.ic_last_error(buf, 256)
    assert b"ic_subsample" in buf.value
    with pytest.raises(_lib.EngineError):
        _lib.check("pf_plan_create", L.pf_plan_create(0, 0, C.c_float(1.0), C.byref(h)), L)
