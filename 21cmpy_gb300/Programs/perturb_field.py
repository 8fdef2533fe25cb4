"""Drop-in for 21cmpy's Programs/perturb_field.py: the density boxes the excursion set reads.

    python -m 21cmpy_gb300.Programs.perturb_field [-z 12] [-d IO_DIR] [--linear | --zeldovich]

Same inputs and outputs as the reference (perturb_field.py:39-148), under IO_DIR/Boxes:

* linear (EVOLVE_DENSITY_LINEARLY): ``smoothed_deltax_z0.00_{HII_DIM}_{L}Mpc.npy`` (or the 21cmFAST
  box of that name) times D(z);
* Zel'dovich: ``deltax_z0.00_{DIM}_{L}Mpc.npy`` moved by ``v{x,y,z}overddot_{HII_DIM}_{L}Mpc.npy``
  times (D(z) - D(INITIAL_REDSHIFT)) / BOX_LEN onto the HII_DIM^3 grid (mass / MASS_FACTOR - 1);

both written as ``updated_smoothed_deltax_z{z:.2f}_{HII_DIM}_{L}Mpc.npy``.  After a Zel'dovich move
the velocity boxes at z are recomputed from the DIM^3 density (perturb_field.py:110-125) and written
as ``updated_v{x,y,z}overddot_{HII_DIM}_{L}Mpc.npy`` (cMpc/s).  The compute runs on the GPU
(``pf_evolve_linear``, ``pf_move_mass``, the engine's real FFTs with ``ic_shape`` and
``ic_subsample``); D(z) is the Carroll-Press-Turner growth normalised to 1 at z = 0 (cosmolopy's
``fgrowth``) and dD/dt / D its rate (``dDdtoverD``), computed on the host in double and rounded to
float32 as the reference's np.float32 does.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from .. import cosmology
from . import _common
from ..tocmfastpy import boxio


def _boxes(p) -> str:
    return os.path.join(str(p["IO_DIR"]), "Boxes")


def output_name(z: float, p) -> str:
    """perturb_field.py:50 / :99."""
    return "updated_smoothed_deltax_z{0:.2f}_{1:d}_{2:.0f}Mpc".format(float(z), int(p["HII_DIM"]), float(p["BOX_LEN"]))


def _load(path_npy: str, raw: str):
    try:
        return np.load(path_npy)
    except OSError:
        return boxio.readbox(raw).box_data


def growth(z: float, p) -> np.float32:
    """pb.fgrowth(z, omega_M_0) as float32 (perturb_field.py:44, :83-84)."""
    return np.float32(cosmology.growth_factor(float(z), _common.cosmo_of(p)))


def evolve_linear(z, deltax, *, params=None, device=None, save=True):
    """updated = deltax * D(z) (perturb_field.py:39-50); returns the host array."""
    import torch
    from .. import perturb
    p = _common.params(params)
    d, _ = _common.to_device(deltax, device or torch.device("cuda", torch.cuda.current_device()))
    out = perturb.evolve_linear(d, float(growth(z, p)))
    updated = out.cpu().numpy()
    if save:
        np.save(os.path.join(_boxes(p), output_name(z, p)), updated)
    return updated


def velocity_name(component: str, p) -> str:
    """perturb_field.py:126."""
    return "updated_v{0}overddot_{1:d}_{2:.0f}Mpc".format(component, int(p["HII_DIM"]), float(p["BOX_LEN"]))


def evolve_velocities(z, deltax, *, params=None, device=None, save=True, hii_dim=None):
    """Velocity boxes at z from the DIM^3 density at z = 0 (perturb_field.py:110-125): returns
    {"vx", "vy", "vz"} host arrays of shape HII_DIM^3, in cMpc/s."""
    import torch
    from .. import perturb
    p = _common.params(params)
    hii = int(p["HII_DIM"]) if hii_dim is None else int(hii_dim)
    dev = device or torch.device("cuda", torch.cuda.current_device())
    d, _ = _common.to_device(deltax, dev)
    dim = int(d.shape[0])
    pf = np.float32(p["PIXEL_FACTOR"]) if dim == int(p["DIM"]) and hii == int(p["HII_DIM"]) else \
        np.float32(dim) / np.float32(hii)
    rate = np.float32(cosmology.growth_rate(float(z), _common.cosmo_of(p)))       # perturb_field.py:117
    vs = perturb.updated_velocities(d, hii, float(p["BOX_LEN"]), float(rate), pixel_factor=float(pf))
    out = {k: v.cpu().numpy() for k, v in vs.items()}
    if save:
        q = dict(p, HII_DIM=hii)
        for c in ("x", "y", "z"):
            np.save(os.path.join(_boxes(p), velocity_name(c, q)), out["v" + c])
    return out


def evolve_zeldovich(z, deltax, vx=None, vy=None, vz=None, *, params=None, device=None, save=True,
                     velocities=True):
    """First-order Zel'dovich move of the DIM^3 box onto the HII_DIM^3 grid (perturb_field.py:52-101),
    then, with ``velocities``, the velocity boxes at z (perturb_field.py:110-125, written when
    ``save``).

    vx, vy, vz: the initial-conditions displacement boxes (v / D-dot, HII_DIM^3, box-axis order
    0, 1, 2); read from IO_DIR/Boxes like the reference when not given."""
    import torch
    from .. import perturb
    p = _common.params(params)
    hii, L = int(p["HII_DIM"]), float(p["BOX_LEN"])
    dim = int(np.asarray(deltax).shape[0]) if not isinstance(deltax, torch.Tensor) else int(deltax.shape[0])
    if L > dim:
        print("perturb_field: WARNING: Resolution is likely too low for accurate evolved density fields",
              file=sys.stderr)
    vs = []
    for name, v in (("x", vx), ("y", vy), ("z", vz)):
        if v is None:
            v = np.load(os.path.join(_boxes(p), "v{0}overddot_{1:d}_{2:.0f}Mpc.npy".format(name, hii, L)))
        vs.append(v)
    hii = int(vs[0].shape[0])
    fg = growth(z, p)
    fg0 = growth(float(p["INITIAL_REDSHIFT"]), p)
    disp = np.float32((fg - fg0) / np.float32(p["BOX_LEN"]))            # perturb_field.py:91-93
    dev = device or torch.device("cuda", torch.cuda.current_device())
    d, _ = _common.to_device(deltax, dev)
    v3 = [_common.to_device(v, dev)[0] for v in vs]
    if dim == int(p["DIM"]):
        pf, mf = np.float32(p["PIXEL_FACTOR"]), np.float32(p["MASS_FACTOR"])
    else:                                     # INIT_PARAMS.py:7-8 for the box actually given
        pf = np.float32(dim) / np.float32(hii)
        mf = np.float32(pf ** 3.0)
    plan = perturb.PerturbPlan(dim, hii, pixel_factor=float(pf), device=d.device)
    try:
        out = plan.move_mass(d, *v3, init_growth=float(fg0), disp_scale=float(disp), mass_factor=float(mf))
        updated = out.cpu().numpy()
    finally:
        plan.close()
    if save:
        np.save(os.path.join(_boxes(p), output_name(z, dict(p, HII_DIM=hii))), updated)
    if velocities:
        from ..engine import supported_sizes
        if dim in supported_sizes():
            evolve_velocities(z, d, params=params, device=dev, save=save, hii_dim=hii)
        else:
            print("perturb_field: WARNING: no velocity boxes: the GPU FFT has no {0}^3 size (supported: {1})"
                  .format(dim, supported_sizes()), file=sys.stderr)
    return updated


def run(z, *, params=None, device=None, linear=None):
    """perturb_field.py:115-143: pick the evolution by EVOLVE_DENSITY_LINEARLY and read its inputs."""
    p = _common.params(params)
    lin = bool(p["EVOLVE_DENSITY_LINEARLY"]) if linear is None else bool(linear)
    hii, dim, L = int(p["HII_DIM"]), int(p["DIM"]), float(p["BOX_LEN"])
    if lin:
        name = "smoothed_deltax_z0.00_{0:d}_{1:.0f}Mpc".format(hii, L)
        deltax = _load(os.path.join(_boxes(p), name + ".npy"), os.path.join(_boxes(p), name))
        return evolve_linear(z, deltax, params=params, device=device)
    name = "deltax_z0.00_{0:d}_{1:.0f}Mpc".format(dim, L)
    deltax = _load(os.path.join(_boxes(p), name + ".npy"), os.path.join(_boxes(p), name))
    return evolve_zeldovich(z, deltax, params=params, device=device)


def parser():
    ap = argparse.ArgumentParser(prog="perturb_field")
    ap.add_argument("-z", "--redshift", type=float, default=12.0)
    ap.add_argument("-d", "--dir", default=None, help="IO_DIR (the Boxes folder lives under it)")
    g = ap.add_mutually_exclusive_group()
    g.add_argument("--linear", dest="linear", action="store_true", default=None)
    g.add_argument("--zeldovich", dest="linear", action="store_false")
    return ap


def main(argv=None):
    a = parser().parse_args(argv)
    params = {"IO_DIR": a.dir} if a.dir else None
    run(a.redshift, params=params, linear=a.linear)
    return 0


if __name__ == "__main__":
    sys.exit(main())
