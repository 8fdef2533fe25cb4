"""One call for find_HII_bubbles.run followed by delta_T.run on the same box, without files.

``simulate_box`` uploads the density once, runs the excursion-set loop, the brightness
temperature and its power spectrum on the GPU, and copies x_HI, delta_T and P(k) back.  Host
inputs and outputs may be numpy arrays or (ideally pinned) torch CPU tensors; device tensors are
used in place.
"""
from __future__ import annotations

import numpy as np

from .. import cosmology, schedule
from . import _common


def simulate_box(deltax, param_dict, Z=None, fil=0, update=0, LE=False, *, params=None,
                 num_bins=None, ref_compat=False, xH_out=None, dT_out=None, device=None):
    """x_HI, delta_T and the binned P(k) of one density box.

    Returns a dict with ``xH``, ``dT`` (boxes in the caller's container type, or written into
    xH_out / dT_out), ``nf`` (mean x_HI), ``ave`` (mean delta_T, mK), ``K``, ``k_ave``,
    ``ps_ave``, ``count`` and ``n_radii``.
    """
    import torch
    p = _common.params(params)
    n = int(np.shape(deltax)[0])
    box_len = float(param_dict["BoxSize"])
    if Z is None:
        Z = param_dict["z"]
    setup = _common.ionize_setup(n, box_len, Z, p, fil=fil, update=update, LE=LE, ref_compat=ref_compat)
    nb = int(num_bins if num_bins is not None else p["NUM_BINS"])
    edges = schedule.pk_edges(n, box_len, nb)
    c = cosmology.brightness_temperature_factor(float(Z), _common.cosmo_of(p))
    plan = _common.plan_for(n, box_len, setup.n_radii, device)
    with torch.cuda.device(plan.device):
        d, kind = _common.to_device(deltax, plan.device)
        xh, nf = plan.run(d, setup, output="xH")
        dT, ave = plan.delta_T(xh, d, c)
        pk = plan.power_spectrum(dT, ave, edges, dimensional=bool(p["DIMENSIONAL_T_POWER_SPEC"]))
        scalars = torch.stack([nf.reshape(()), ave.reshape(())])
        xh_h = _common.to_host(xh, kind, xH_out)
        dT_h = _common.to_host(dT, kind, dT_out)
        pk_h = pk.cpu().numpy().astype(np.float64)
        nf_h, ave_h = (float(v) for v in scalars.cpu().numpy())
    return {"xH": xh_h, "dT": dT_h, "nf": nf_h, "ave": ave_h, "K": edges, "k_ave": pk_h[1],
            "ps_ave": pk_h[0], "count": pk_h[2], "n_radii": setup.n_radii}
