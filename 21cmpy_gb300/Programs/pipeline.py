"""One call for find_HII_bubbles.run followed by delta_T.run on the same box, without files.

``simulate_box`` uploads the density once, runs the excursion-set loop, the brightness
temperature and its power spectrum on the GPU, and copies x_HI, delta_T and P(k) back.  Host
inputs and outputs may be numpy arrays or (ideally pinned) torch CPU tensors; device tensors are
used in place.  ``simulate_sweep`` does the same for a list of boxes with the host <-> device
copies of neighbouring boxes overlapped with the compute.
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


MAX_LANES = 4


def lane_slot(i: int, lanes: int):
    """(lane, device slot) of box i when ``lanes`` boxes run side by side: box i runs on lane
    i mod lanes, and each lane alternates between two slots, so a slot is reused by box i + 2 lanes
    and never by a box that can still be in flight beside it."""
    lane = i % lanes
    return lane, 2 * lane + ((i // lanes) & 1)


def simulate_sweep(boxes, param_dict, Zs, fil=0, update=0, LE=False, *, params=None, num_bins=None,
                   ref_compat=False, xH_outs=None, dT_outs=None, device=None, lanes=3):
    """``simulate_box`` for many boxes of one size, with the copies overlapped with the compute and
    ``lanes`` boxes computed side by side.

    boxes: host (N, N, N) float32 boxes (pinned torch CPU tensors for the copies to overlap; numpy
    arrays are pinned here first); Zs: their redshifts.  Box i runs on lane i mod lanes (a plan and
    a stream of its own); while it runs, later boxes are copied in and earlier boxes' x_HI and
    delta_T are copied out on their own streams.  Each lane reuses two device slots per box
    quantity, guarded by CUDA events.  x_HI and delta_T go to xH_outs / dT_outs (host tensors;
    allocated pinned when not given).  Returns a list of dicts as ``simulate_box`` does, with the
    boxes as torch CPU tensors; results are identical to box-by-box ``simulate_box``.
    """
    import torch
    if int(lanes) < 1:
        raise ValueError("lanes must be >= 1")
    if len(boxes) != len(Zs):
        raise ValueError("one redshift per box")
    if not boxes:
        return []
    p = _common.params(params)
    boxes = [b if isinstance(b, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(b, np.float32)).pin_memory()
             for b in boxes]
    n = int(boxes[0].shape[0])
    if any(tuple(b.shape) != (n, n, n) or b.dtype != torch.float32 or b.is_cuda for b in boxes):
        raise ValueError("boxes must be host float32 (N, N, N) tensors or arrays of one size")
    box_len = float(param_dict["BoxSize"])
    nb = int(num_bins if num_bins is not None else p["NUM_BINS"])
    edges = schedule.pk_edges(n, box_len, nb)
    cosmo = _common.cosmo_of(p)
    setups = [_common.ionize_setup(n, box_len, float(z), p, fil=fil, update=update, LE=LE, ref_compat=ref_compat)
              for z in Zs]
    consts = [cosmology.brightness_temperature_factor(float(z), cosmo) for z in Zs]
    nbox = len(boxes)
    # at most MAX_LANES plans of a size: the plan cache must hold them all (four lanes measured no
    # faster than three at 256^3)
    K = min(int(lanes), nbox, MAX_LANES)
    radii = max(s.n_radii for s in setups)
    plans = [_common.plan_for(n, box_len, radii, device, lane=k) for k in range(K)]
    dev = plans[0].device
    xH_outs = xH_outs or [torch.empty((n, n, n), dtype=torch.float32).pin_memory() for _ in range(nbox)]
    dT_outs = dT_outs or [torch.empty((n, n, n), dtype=torch.float32).pin_memory() for _ in range(nbox)]
    with torch.cuda.device(dev):
        main = torch.cuda.current_stream(dev)
        comps = [torch.cuda.Stream(dev) for _ in range(K)]
        s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        fork = torch.cuda.Event()
        fork.record(main)
        for st_ in comps + [s_in, s_out]:
            st_.wait_event(fork)
        d_in = [torch.empty((n, n, n), dtype=torch.float32, device=dev) for _ in range(2 * K)]
        d_xh = [torch.empty_like(d_in[0]) for _ in range(2 * K)]
        d_dT = [torch.empty_like(d_in[0]) for _ in range(2 * K)]
        nf = torch.empty(nbox, dtype=torch.float32, device=dev)
        ave = torch.empty(nbox, dtype=torch.float32, device=dev)
        pk = torch.empty((nbox, 3, len(schedule.pk_k2_thresholds(n, box_len, np.asarray(edges)))),
                         dtype=torch.float32, device=dev)
        ev_in = [torch.cuda.Event() for _ in range(nbox)]
        ev_comp = [torch.cuda.Event() for _ in range(nbox)]
        ev_out = [torch.cuda.Event() for _ in range(nbox)]
        for i in range(nbox):
            lane, slot = lane_slot(i, K)                      # box i - 2K used this slot last
            comp, plan = comps[lane], plans[lane]
            with torch.cuda.stream(s_in):
                if i >= 2 * K:
                    s_in.wait_event(ev_comp[i - 2 * K])       # box i - 2K no longer reads this slot
                d_in[slot].copy_(boxes[i], non_blocking=True)
                ev_in[i].record(s_in)
            comp.wait_event(ev_in[i])
            if i >= 2 * K:
                comp.wait_event(ev_out[i - 2 * K])            # box i - 2K's outputs have left the slot
            plan.run(d_in[slot], setups[i], out=d_xh[slot], nf=nf[i:i + 1], output="xH", stream=comp)
            plan.delta_T(d_xh[slot], d_in[slot], consts[i], out=d_dT[slot], ave=ave[i:i + 1], stream=comp)
            plan.power_spectrum(d_dT[slot], ave[i:i + 1], edges, dimensional=bool(p["DIMENSIONAL_T_POWER_SPEC"]),
                                out=pk[i], stream=comp)
            ev_comp[i].record(comp)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_comp[i])
                xH_outs[i].copy_(d_xh[slot], non_blocking=True)
                dT_outs[i].copy_(d_dT[slot], non_blocking=True)
                ev_out[i].record(s_out)
        for st_ in comps + [s_out]:
            main.wait_stream(st_)
        nf_h, ave_h, pk_h = nf.cpu().numpy(), ave.cpu().numpy(), pk.cpu().numpy().astype(np.float64)
    return [{"xH": xH_outs[i], "dT": dT_outs[i], "nf": float(nf_h[i]), "ave": float(ave_h[i]), "K": edges,
             "k_ave": pk_h[i, 1], "ps_ave": pk_h[i, 0], "count": pk_h[i, 2], "n_radii": setups[i].n_radii}
            for i in range(nbox)]
