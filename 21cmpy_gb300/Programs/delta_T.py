"""Drop-in for 21cmpy's Programs/delta_T.py on the GB300 engine.

* ``run(xHfile=None, IO_DIR=None)`` -> ``(K, k_ave, ps_ave)`` (delta_T.py:32-103): loads the x_HI
  box and its density, writes ``delta_T_no_halos_z..._aveTb{ave:.2f}_{N}_{L}Mpc.npy`` and returns
  the spherically binned power spectrum of the normalised brightness temperature;
* ``compute(xH, deltax, Z, box_len)`` -> the same on arrays, without files;
* ``python -m 21cmpy_gb300.Programs.delta_T [-d DIR] <xH file>`` (delta_T.py:106-111).

The P(k) is the estimator the reference's ``pbox_kernel`` intends (delta_T.cu:5-29): modes are
binned by the first edge >= |k|, per-bin means of k^3 |g_k|^2 / (2 pi^2 V) and of |k| are
returned, and the k = 0 mode is excluded.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from .. import cosmology, schedule
from ..tocmfastpy import boxio
from . import _common


def compute(xH, deltax, Z, box_len, *, params=None, device=None, num_bins=None, edge_dim=None,
            dT_out=None):
    """delta_T box, its mean and binned P(k) from x_HI and density boxes.

    Returns ``(dT, ave, K, k_ave, ps_ave)``; dT comes back in the input's container type.
    """
    import torch
    p = _common.params(params)
    n = int(np.shape(xH)[0])
    nb = int(num_bins if num_bins is not None else p["NUM_BINS"])
    plan = _common.plan_for(n, float(box_len), 1, device)
    x, kind = _common.to_device(xH, plan.device)
    d, _ = _common.to_device(deltax, plan.device)
    c = cosmology.brightness_temperature_factor(float(Z), _common.cosmo_of(p))
    edges = schedule.pk_edges(n, float(box_len), nb, edge_dim)
    with torch.cuda.device(plan.device):
        dT, ave = plan.delta_T(x, d, c)
        pk = plan.power_spectrum(dT, ave, edges, dimensional=bool(p["DIMENSIONAL_T_POWER_SPEC"]))
        pk_h = pk.cpu().numpy().astype(np.float64)
        ave_h = float(ave.item())
        dT_h = _common.to_host(dT, kind, dT_out)
    return dT_h, ave_h, edges, pk_h[1], pk_h[0]


def _density_for(io_dir, Z, n, L):
    # the reference looks for z0{Z:.2f} (delta_T.py:56); perturb_field writes z{Z:.2f}
    # (perturb_field.py:50) and 21cmFAST z{Z:06.2f}: accept all three
    names = [f"updated_smoothed_deltax_z0{Z:.2f}_{n:d}_{L:.0f}Mpc.npy",
             f"updated_smoothed_deltax_z{Z:.2f}_{n:d}_{L:.0f}Mpc.npy",
             f"updated_smoothed_deltax_z{Z:06.2f}_{n:d}_{L:.0f}Mpc.npy"]
    for nm in names:
        f = os.path.join(io_dir, "Boxes", nm)
        if os.path.exists(f):
            return np.load(f)
    raw = os.path.join(io_dir, "Boxes", names[0][:-4].replace(f"_{n:d}_", f"_{2 * n:d}_"))
    if os.path.exists(raw):
        return boxio.readbox(raw).box_data[:n, :n, :n]
    raise FileNotFoundError(f"no density box for z={Z}, {n}^3, {L:.0f} Mpc under {io_dir}/Boxes")


def run(xHfile=None, IO_DIR=None, *, params=None):
    """delta_T.run: read x_HI + density, save the delta_T box, return (K, k_ave, ps_ave)."""
    p = _common.params(params)
    io_dir = IO_DIR if IO_DIR is not None else str(p["IO_DIR"])
    if xHfile is None:
        raise ValueError("xHfile is required (the reference's default lookup uses an undefined Z)")
    if xHfile.endswith(".npy"):
        xH = np.load(xHfile)
        pd = boxio.parse_filename(os.path.splitext(xHfile)[0])
    else:
        b = boxio.readbox(xHfile)
        xH, pd = b.box_data, b.param_dict
    Z = pd["z"]
    n = int(pd["dim"])
    L = float(np.float32(pd["BoxSize"]))
    deltax = _density_for(io_dir, Z, n, L)
    dT, ave, K, k_ave, ps_ave = compute(xH, deltax, Z, L, params=params)
    os.makedirs(os.path.join(io_dir, "Boxes"), exist_ok=True)
    name = "delta_T_no_halos_z{0:.2f}_nf{1:f}_useTs{2:d}_zetaX{3:.1e}_TvirminX{4:.1e}_aveTb{5:.2f}_{6:d}_{7:d}Mpc.npy".format(
        Z, pd.get("nf", 0.0), int(p["USE_TS_IN_21CM"]), pd.get("eff", float(p["ZETA"])),
        float(p["ION_Tvir_MIN"]), ave, n, int(L))
    np.save(os.path.join(io_dir, "Boxes", name), dT)
    return K, k_ave, ps_ave


def main(argv=None):
    p = _common.params()
    o = argparse.ArgumentParser(prog="delta_T")
    o.add_argument("-d", "--dir", dest="DIR", default=str(p["IO_DIR"]))
    o.add_argument("-i", "--inter", dest="INTERACTIVE", action="store_true")
    o.add_argument("args", nargs=1)
    opts = o.parse_args(argv)
    K, k_ave, ps = run(opts.args[0], opts.DIR)
    for k, kv, v in zip(K, k_ave, ps):
        print(f"{k:.6e} {kv:.6e} {v:.6e}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
