"""21cmFAST box file names and raw boxes (tocmfastpy/boxio.py:30-293, Programs/IO_utils.py:18-26).

The file name carries the box parameters (``_z``, ``_nf``, ``_eff``, ``_HIIfilter``,
``_RHIImax``, ``_<HIIdim>_<L>Mpc``, ``_L``); raw boxes are float32 C-order, optionally with
FFTW's in-place padding along the last axis.
"""
from __future__ import annotations

import fnmatch
import os
import re

import numpy as np


class BoxFormatError(ValueError):
    """Malformed box file (the reference prints and calls sys.exit, boxio.py:240-244)."""


class Box:
    """A box with its parameters (tocmfastpy/Box.py:7-31)."""

    def __init__(self, box_data=None, param_dict=None):
        self.box_data = box_data
        self.param_dict = param_dict or {}
        self.dim = self.param_dict.get("dim")
        self.z = self.param_dict.get("z", -1)
        self.init = box_data is not None

    def setBox(self, box_data, param_dict):  # noqa: N802 (the reference's name, Box.py:24-31)
        self.box_data = box_data
        self.param_dict = param_dict
        self.dim = param_dict["dim"]
        self.z = param_dict["z"]
        self.init = True


_TYPES = [("updated_smoothed_deltax", "density"), ("xH_nohalos", "xh"), ("delta_T", "deltaT"),
          ("updated_vx", "vx"), ("updated_vy", "vy"), ("updated_vz", "vz"),
          ("smoothed_deltax", "density"), ("vxoverddot", "vx"), ("vyoverddot", "vy"),
          ("vzoverddot", "vz"), ("deltax", "init_x"), ("deltak", "init_k")]


def validate_box_type(prefix: str) -> str:
    """Box type from the file-name prefix (boxio.py:149-194)."""
    for tag, kind in _TYPES:
        if prefix.startswith(tag):
            return kind
    return prefix


def parse_filename(filepath: str) -> dict:
    """Parameters encoded in a 21cmFAST file name (boxio.py:52-146)."""
    base, filename = os.path.split(filepath)
    d: dict = {}
    if not filename:
        d["type"] = False
        d["z"] = False
        return d
    d["filename"] = filename
    d["basedir"] = base
    m = re.search(r"([a-zA-Z]+_)+", filename)
    if m:
        d["type"] = validate_box_type(m.group())
    for key, pat, conv in [("nf", r"_nf([0-9.]+)", float), ("eff", r"_eff([0-9.]+)", float),
                           ("HIIfilter", r"_HIIfilter([0-9]+)", int), ("Mmin", r"_Mmin([0-9.e+-]+)", float),
                           ("RHIIfilter", r"_RHIImax([0-9.]+)", float)]:
        m = re.search(pat, filename)
        if m:
            d[key] = conv(_strip_dot(m.group(1)) if conv is float else m.group(1))
    m = re.search(r"_z([0-9.]+)", filename)
    d["z"] = float(_strip_dot(m.group(1))) if m else 0.0
    m = re.search(r"_([0-9]+)_([0-9]+)Mpc", filename)
    if m:
        d["HIIdim"] = int(m.group(1))
        d["dim"] = int(m.group(1))
        d["BoxSize"] = int(m.group(2))
    m = re.search(r"_Iter([0-9]+)", filename)
    d["Iteration"] = int(m.group(1)) if m else 0
    m = re.search(r"_L([0-9]+)", filename)
    if m:
        d["BoxSize"] = int(m.group(1))
    return d


def _strip_dot(s: str) -> str:
    # "8.00_" style matches can end in a trailing '.' before the extension
    return s[:-1] if s.endswith(".") else s


def trim_box(box: np.ndarray) -> np.ndarray:
    """Drop FFTW padding along the last axis (boxio.py:198-206)."""
    if box.shape[2] > box.shape[0]:
        return box[:, :, : box.shape[0]]
    return box


def open_box(filename: str, dim: int) -> np.ndarray:
    """Raw float32 box of side dim, or a padded / differently sized cubic one (boxio.py:209-253)."""
    data = np.fromfile(filename, dtype=np.float32)
    size = dim ** 3
    if data.size == size:
        shape = (dim, dim, dim)
    else:
        root = int(round(data.size ** (1.0 / 3.0)))
        for r in (root - 1, root, root + 1):
            if r > 0 and r ** 3 == data.size:
                shape = (r, r, r)
                break
            if r > 0 and r * r * 2 * (r // 2 + 1) == data.size:
                shape = (r, r, 2 * (r // 2 + 1))
                break
        else:
            raise BoxFormatError(f"{filename}: {data.size} floats is neither a cubic box nor an "
                                 f"FFTW-padded one (expected dim {dim})")
    return trim_box(data.reshape(shape))


def readbox(filename: str, quiet: bool = False) -> Box:
    """Read a 21cmFAST box and its file-name parameters (boxio.py:30-49); prints the parameters
    unless quiet, as the reference does."""
    d = parse_filename(filename)
    if not quiet:
        print(d)
    if "HIIdim" not in d:
        raise BoxFormatError(f"{filename}: no _<dim>_<L>Mpc field in the file name")
    return Box(open_box(filename, d["HIIdim"]), d)


def save_box(filename: str, box: np.ndarray) -> None:
    np.asarray(box, dtype=np.float32).tofile(filename)


def find_run_boxes(filename: str) -> list:
    """Every file of the run that ``filename`` belongs to (boxio.py:272-293): the files in its
    directory whose names start with its leading alphanumeric tag and carry its
    ``_<HIIdim>_<BoxSize>Mpc`` field, sorted by name."""
    d = parse_filename(filename)
    base, fname = os.path.split(filename)
    if "HIIdim" not in d:
        raise BoxFormatError(f"{filename}: no _<dim>_<L>Mpc field in the file name")
    m = re.match(r"[a-zA-Z0-9]+", fname)
    if not m:
        raise BoxFormatError(f"{filename}: the file name has no leading tag")
    tag, field = m.group(), "_{0}_{1}Mpc".format(d["HIIdim"], d["BoxSize"])
    return sorted(os.path.join(base, f) for f in os.listdir(base or ".") if f.startswith(tag) and field in f)


def find_files(directory: str, pattern: str = "*") -> np.ndarray:
    """Recursively find files matching pattern, sorted (Programs/IO_utils.py:18-26)."""
    files = []
    for root, _dirs, names in os.walk(directory):
        files.extend(os.path.join(root, f) for f in fnmatch.filter(names, pattern))
    if not files:
        raise FileNotFoundError(f"no files matching {pattern!r} under {directory}")
    return np.sort(files)
