"""Drop-in for 21cmpy's Programs/find_HII_bubbles.py on the GB300 engine.

Same entry points as the reference:

* ``conv_bubbles(deltax, param_dict, Z=None, scale=None, fil=1, update=0, LE=False,
  visualize=0, quiet=False)`` -> ionised-fraction box (find_HII_bubbles.py:17-193);
* ``run(opts, args)`` -> reads the density file, writes the x_HI box
  ``xH_nohalos_z{Z:.2f}_nf{nf:f}_eff{ZETA:.1f}_HIIfilter{f}_Tvirmin{T:.1f}_RHIImax{R}_{N}_{L}Mpc.npy``
  (l.195-232);
* ``python -m 21cmpy_gb300.Programs.find_HII_bubbles [-d DIR] [-f FILTER] [-u UPDATE] [-z Z]
  [-v VIS] [-q] [-i] <density file>`` (l.235-246).

Parameters come from ``Parameter_files/INIT_PARAMS`` (ZETA, ION_Tvir_MIN, R_BUBBLE_MAX,
R_BUBBLE_MIN, DELTA_R_FACTOR, COSMO, ...) or from ``params=`` overrides.  The radius loop runs on
the CUDA engine; there is no CPU path.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from ..tocmfastpy import boxio
from . import _common


def conv_bubbles(deltax, param_dict, Z=None, scale=None, fil=1, update=0, LE=False, visualize=0,
                 quiet=False, *, params=None, ref_compat=False, device=None, output="ionized", out=None):
    """Excursion-set ionisation field of one density box (find_HII_bubbles.py:17-193).

    deltax: (N, N, N) density contrast (numpy array, host or device torch tensor).
    param_dict: ``boxio.parse_filename`` output (needs BoxSize and HIIdim).
    Z: redshift; fil: 0 real-space top-hat, 1 k-space top-hat, 2 Gaussian; update: 0 centre
    pixel, 1 sphere painting; LE: density already linear at z = 0 (no growth rescale, no mean
    normalisation).  ref_compat=True reproduces the reference kernels' quirks (filter
    fall-through, sphere radius in Mpc used as cells, clamped spheres).
    Returns the ionised fraction (``output="xH"``: 1 - ionised) in the input's container type.
    """
    import torch
    p = _common.params(params)
    n = int(np.shape(deltax)[0])
    if tuple(np.shape(deltax)) != (n, n, n):
        raise ValueError(f"density box must be cubic, got {tuple(np.shape(deltax))}")
    if Z is None:
        Z = param_dict["z"] if "z" in param_dict else param_dict["Z"]
    box_len = float(param_dict["BoxSize"])
    if "HIIdim" in param_dict and int(param_dict["HIIdim"]) != n:
        raise ValueError(f"param_dict HIIdim={param_dict['HIIdim']} does not match the box ({n})")
    setup = _common.ionize_setup(n, box_len, Z, p, fil=fil, update=update, LE=LE, scale=scale,
                                 ref_compat=ref_compat)
    if not quiet:
        print(f"Using filter_type {int(fil)}; {setup.n_radii} radii from R={float(setup.steps[0].R)} Mpc")
    plan = _common.plan_for(n, box_len, setup.n_radii, device)
    d, kind = _common.to_device(deltax, plan.device)
    with torch.cuda.device(plan.device):
        res, _nf = plan.run(d, setup, output="xH" if output == "xH" else "ionized")
        result = _common.to_host(res, kind, out)
    if visualize:
        _dump_slices(d, res, visualize)
    return result


def _dump_slices(d, res, visualize):
    # the reference draws matplotlib slices (l.94-111, 178-186); without a graphics stack the
    # mid-plane slices are written as .npy files instead
    if int(visualize) == 2:
        os.makedirs("tmp", exist_ok=True)
        mid = d.shape[0] // 2
        np.save(os.path.join("tmp", "density_slice.npy"), d[mid].float().cpu().numpy())
        np.save(os.path.join("tmp", "ionization_slice.npy"), res[mid].float().cpu().numpy())


def output_name(Z, nf, p, fil, n, box_len) -> str:
    return "xH_nohalos_z{0:.2f}_nf{1:f}_eff{2:.1f}_HIIfilter{3:d}_Tvirmin{4:.1f}_RHIImax{5:d}_{6:d}_{7:d}Mpc.npy".format(
        float(Z), float(nf), float(p["ZETA"]), int(fil), float(p["ION_Tvir_MIN"]), int(p["R_BUBBLE_MAX"]),
        int(n), int(box_len))


def run(opts, args, params=None):
    """Read the density box named in args[0], ionise it and save x_HI (l.195-232)."""
    if len(args) < 1:
        raise Exception("Must specify density box input!")
    fname = args[0]
    if fname.endswith("npy"):
        param_dict = boxio.parse_filename(fname)
        d1 = np.load(fname)
    else:
        b1 = boxio.readbox(fname)
        d1 = b1.box_data[:256, :256, :256]          # l.211
        param_dict = b1.param_dict
    if not param_dict["filename"].startswith("updated"):
        Z = float(opts.Z)
        LE = True
    else:
        Z = param_dict["z"]
        LE = False
    p = _common.params(params)
    fil = int(opts.FILTER_TYPE)
    ion = conv_bubbles(d1, param_dict, Z, fil=fil, update=int(opts.UPDATE_TYPE), LE=LE,
                       visualize=int(opts.VISUAL), quiet=bool(opts.QUIET), params=params)
    nf = 1.0 - float(np.mean(ion, dtype=np.float64))
    outname = output_name(Z, nf, p, fil, ion.shape[0], param_dict["BoxSize"])
    os.makedirs(opts.DIR, exist_ok=True)
    if not opts.QUIET:
        print("saving", outname)
    np.save(os.path.join(opts.DIR, outname), (np.float32(1.0) - ion).astype(np.float32))
    return ion


def parser():
    p = _common.params()
    o = argparse.ArgumentParser(prog="find_HII_bubbles")
    o.add_argument("-d", "--dir", dest="DIR", default=os.path.join(str(p["IO_DIR"]), "Boxes"))
    o.add_argument("-f", "--filt", dest="FILTER_TYPE", type=int, default=int(p["HII_FILTER"]),
                   help="0: rtophat; 1: ktophat, 2: Gaussian")
    o.add_argument("-u", "--upd", dest="UPDATE_TYPE", type=int, default=int(p["FIND_BUBBLE_ALGORITHM"]),
                   help="0: center pixel, 1: sphere painting")
    o.add_argument("-z", "--reds", dest="Z", type=float, default=12.0,
                   help="redshift, needed if using a linear density field at z=0")
    o.add_argument("-v", "--vis", dest="VISUAL", type=int, default=0,
                   help="0: none, 2: save mid-plane slices as .npy")
    o.add_argument("-q", "--qui", dest="QUIET", action="store_true")
    o.add_argument("-i", "--inter", dest="INTERACTIVE", action="store_true")
    o.add_argument("args", nargs="*")
    return o


def main(argv=None):
    opts = parser().parse_args(argv)
    run(opts, opts.args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
