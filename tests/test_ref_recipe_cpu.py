"""The second oracle's build recipe (oracle/build_ref.py), checked on the host: the reference's
templating with the reference's formatting of the values, and an nvcc build of the result."""
import shutil

import numpy as np
import pytest

from oracle import build_ref


@pytest.fixture(scope="module")
def staged():
    build_ref.stage()
    if not build_ref.available():
        pytest.skip("no reference checkout here and nothing staged under oracle/_ref")
    return True


def test_templating_fills_every_placeholder_as_the_reference_prints_it(staged):
    text = build_ref.render(13.123456789, 30.0, 100.0)
    assert "float deltac = 13.123456789;" in text            # find_bubbles.cu:54
    assert "1/30.0" in text and "* 30.0" in text              # find_bubbles.cu:70, 154-156
    dk = str(np.float32(2 * np.pi / np.float32(100.0)))
    assert f"(k-w)*{dk}" in text and f"i*{dk}" in text         # find_bubbles.cu:22-24
    assert "%(" not in text
    # the staged file is the reference's own source, byte for byte (only templating differs)
    assert build_ref.STAGED.read_text() % {"DELTAC": "13.123456789", "RMIN": "0.5", "ZETA": "30.0",
                                           "DELTAK": dk} == text


def test_reference_kernels_build_for_sm_103a(staged):
    if not (shutil.which("nvcc") or build_ref.Path("/usr/local/cuda/bin/nvcc").exists()):
        pytest.skip("no nvcc")
    lib = build_ref.build(11.0, 40.0, 600.0)
    assert lib.is_file() and lib.stat().st_size > 0
    assert build_ref.build(11.0, 40.0, 600.0) == lib            # cached by content
