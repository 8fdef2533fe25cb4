"""Recipe for the second oracle: the reference's own excursion-set kernels -- TEST INFRASTRUCTURE ONLY.

Only the parity tests use what this builds; the product never builds, loads or calls it.

The reference compiles ``Programs/find_bubbles.cu`` at run time with PyCUDA after filling its
``%(DELTAC)s``-style placeholders from Python (find_HII_bubbles.py:63-70).  This recipe does the
same steps without PyCUDA:

* ``stage()`` copies ``Programs/find_bubbles.cu`` verbatim from a checkout of the reference
  (``--reference DIR``, the ``ES_REFERENCE_DIR`` environment variable, else ``/root/reference``)
  into ``oracle/_ref/`` (git-ignored), the only file it reads there.  The copy travels with the
  repository to a GPU machine that has no checkout.
* ``render()`` applies the reference's own templating, ``source % {...}``, with the values
  formatted as the reference formats them: ``DELTAC`` a Python float (``repr``, the shortest
  round-trip digits), ``ZETA`` a Python float (``ZETA = 40.`` in INIT_PARAMS.py:20 gives
  ``40.0``), ``DELTAK`` the string of ``np.float32(2 pi / np.float32(BOX_LEN))``
  (INIT_PARAMS.py:9-10), ``RMIN`` unused by the kernels.
* ``build()`` compiles the rendered copy, unmodified, with ``oracle/ref_launch.cu`` (C
  launchers, 8x8x8 blocks as INIT_PARAMS.py:49) and ``oracle/ref_shim/`` on the include path
  (a ``pycuda::complex`` alias and an empty ``texture`` template, so line 9's legacy texture
  declaration stands as an unused host object): nvcc for sm_103a, one shared library per
  parameter set under ``oracle/_ref/build/``, cached by the hash of what it compiles.

Run ``python oracle/build_ref.py`` in a container with the reference checkout to stage the copy.
"""
from __future__ import annotations

import argparse
import hashlib
import math
import os
import platform
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
STAGED = OUT / "find_bubbles.cu"
LAUNCH = HERE / "ref_launch.cu"
SHIM = HERE / "ref_shim"
DEFAULT_REFERENCE = "/root/reference"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def reference_dir(arg: str | None = None) -> Path | None:
    for cand in (arg, os.environ.get("ES_REFERENCE_DIR"), DEFAULT_REFERENCE):
        if cand and (Path(cand) / "Programs" / "find_bubbles.cu").is_file():
            return Path(cand)
    return None


def stage(ref: str | None = None) -> Path | None:
    """Copies the reference's find_bubbles.cu into oracle/_ref/ when a checkout is present."""
    src = reference_dir(ref)
    if src is None:
        return STAGED if STAGED.is_file() else None
    OUT.mkdir(exist_ok=True)
    data = (src / "Programs" / "find_bubbles.cu").read_bytes()
    if not STAGED.is_file() or STAGED.read_bytes() != data:
        tmp = STAGED.with_suffix(".tmp")
        tmp.write_bytes(data)
        os.replace(tmp, STAGED)
    return STAGED


def available() -> bool:
    return STAGED.is_file()


def deltak_text(box_len: float) -> str:
    """DELTA_K = np.float32(2*np.pi/BOX_LEN) with BOX_LEN = np.float32(L) (INIT_PARAMS.py:9-10)."""
    return str(np.float32(2 * math.pi / np.float32(box_len)))


def render(delta_c: float, zeta: float, box_len: float, r_min: float = 0.5) -> str:
    """find_HII_bubbles.py:63-69: the kernel source with its placeholders filled."""
    if not available():
        raise FileNotFoundError("the reference's find_bubbles.cu is not staged under oracle/_ref "
                                "(run oracle/build_ref.py where a reference checkout exists)")
    source = STAGED.read_text()
    return source % {"DELTAC": repr(float(delta_c)), "RMIN": repr(float(r_min)),
                     "ZETA": repr(float(zeta)), "DELTAK": deltak_text(box_len)}


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found")
    return path


def build(delta_c: float, zeta: float, box_len: float) -> Path:
    """Compiles the rendered kernels for one parameter set; returns the shared library's path."""
    text = render(delta_c, zeta, box_len)
    key = hashlib.sha256((text + LAUNCH.read_text() + (SHIM / "pycuda-complex.hpp").read_text()
                          + " ".join(ARCH) + platform.machine()).encode()).hexdigest()[:16]
    bdir = OUT / "build"
    bdir.mkdir(parents=True, exist_ok=True)
    lib = bdir / f"refkernels_{key}.so"
    if lib.is_file():
        return lib
    cu = bdir / f"find_bubbles_{key}.cu"
    cu.write_text(text)
    tmp = bdir / f"refkernels_{key}.so.tmp{os.getpid()}"
    cmd = [_nvcc(), *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", f"-I{SHIM}",
           f'-DREF_SOURCE="{cu}"', str(LAUNCH), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"building the reference kernels failed:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description="stage (and test-build) the reference's find_bubbles.cu")
    ap.add_argument("--reference", default=None, help="reference checkout (default: ES_REFERENCE_DIR, /root/reference)")
    ap.add_argument("--no-build", action="store_true", help="stage only")
    args = ap.parse_args()
    path = stage(args.reference)
    if path is None:
        raise SystemExit("no reference checkout found and nothing staged")
    print("staged", path)
    if not args.no_build:
        print("built", build(13.7, 30.0, 100.0))
