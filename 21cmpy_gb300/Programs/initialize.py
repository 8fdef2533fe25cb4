"""Drop-in for 21cmpy's Programs/initialize.py: the initial-conditions boxes.

    python -m 21cmpy_gb300.Programs.initialize [-d IO_DIR] [--seed S]

Writes, under IO_DIR/Boxes, the reference's files (initialize.py:83-109):
``deltax_z0.00_{DIM}_{L}Mpc.npy`` (density at z = 0), ``smoothed_deltax_z0.00_{HII_DIM}_{L}Mpc.npy``
(top-hat smoothed with R = L_FACTOR * BOX_LEN / HII_DIM and subsampled) and
``v{x,y,z}overddot_{HII_DIM}_{L}Mpc.npy`` (displacement per unit growth, smoothed and subsampled),
computed on the GPU (``ic_*`` kernels around the engine's inverse FFT).  DIM must be one of the
engine's FFT sizes.  The random field is drawn as a Hermitian half spectrum from a seeded
generator (the reference's MRG32k3a stream is not reproduced).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import _common


def init(*, params=None, seed: int = 0, device=None, save=True, ref_compat=False) -> dict:
    """initialize.py:33-111; returns the host boxes by their file stems."""
    from ..initial import InitialConditions
    p = _common.params(params)
    dim, hii, L = int(p["DIM"]), int(p["HII_DIM"]), float(p["BOX_LEN"])
    with InitialConditions(dim, hii, L, cosmo=_common.cosmo_of(p), device=device) as ic:
        boxes = ic.generate(seed=seed, ref_compat=ref_compat)
        out = {"deltax_z0.00_{0:d}_{1:.0f}Mpc".format(dim, L): boxes["deltax"].cpu().numpy(),
               "smoothed_deltax_z0.00_{0:d}_{1:.0f}Mpc".format(hii, L): boxes["smoothed"].cpu().numpy()}
        for name in ("x", "y", "z"):
            out["v{0}overddot_{1:d}_{2:.0f}Mpc".format(name, hii, L)] = boxes["v" + name].cpu().numpy()
    if save:
        d = os.path.join(str(p["IO_DIR"]), "Boxes")
        os.makedirs(d, exist_ok=True)
        for stem, arr in out.items():
            np.save(os.path.join(d, stem + ".npy"), arr)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="initialize")
    ap.add_argument("-d", "--dir", default=None, help="IO_DIR (the Boxes folder lives under it)")
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    init(params={"IO_DIR": a.dir} if a.dir else None, seed=a.seed)
    return 0


if __name__ == "__main__":
    sys.exit(main())
