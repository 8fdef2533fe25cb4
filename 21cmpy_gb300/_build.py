"""Builds the engine's shared libraries in-tree with nvcc for sm_103a.

``libes_engine.so``: one object per supported box size (``es_inst.cu`` with ``-DES_N``) plus the
host engine, compiled in parallel and linked into one shared library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libes_engine.so"
SIZES = (16, 32, 48, 64, 96, 128, 160, 256, 512, 1024)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the engine")
    return path


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return proc


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        sorted(INCLUDE.glob("*.h"))


def _stale(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in _sources())


def build(force: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libes_engine.so if any source is newer than it; returns its path."""
    if not force and not _stale(LIB):
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = jobs or min(len(SIZES) + 1, os.cpu_count() or 4)
    units = [([cc, *ARCH, *FLAGS, f"-DES_N={n}", "-c", str(CSRC / "es_inst.cu"), "-o",
               str(BUILD / f"es_inst_{n}.o")], BUILD / f"es_inst_{n}.o") for n in SIZES]
    for unit in ("es_engine", "es_batch", "sg_conv", "sg_tc", "pf", "ic"):
        units.append(([cc, *ARCH, *FLAGS, "-c", str(CSRC / f"{unit}.cu"), "-o", str(BUILD / f"{unit}.o")],
                      BUILD / f"{unit}.o"))
    with cf.ThreadPoolExecutor(jobs) as ex:
        list(ex.map(lambda u: _run(u[0]), units))
    tmp = LIB.with_suffix(".so.tmp")
    _run([cc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in units]])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
