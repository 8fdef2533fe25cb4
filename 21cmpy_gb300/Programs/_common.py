"""Shared host plumbing of the drop-in programs: parameters, plans, host<->device transfers."""
from __future__ import annotations

import collections
import threading

import numpy as np

from .. import cosmology, schedule
from ..Parameter_files import INIT_PARAMS as _P

PARAM_NAMES = ("IO_DIR", "ZETA", "ION_Tvir_MIN", "R_BUBBLE_MAX", "R_BUBBLE_MIN", "DELTA_R_FACTOR",
               "HII_FILTER", "FIND_BUBBLE_ALGORITHM", "COSMO", "NUM_BINS", "DIMENSIONAL_T_POWER_SPEC",
               "USE_TS_IN_21CM", "DIM", "HII_DIM", "BOX_LEN", "PIXEL_FACTOR", "MASS_FACTOR", "INITIAL_REDSHIFT",
               "EVOLVE_DENSITY_LINEARLY")


def params(overrides: dict | None = None) -> dict:
    """INIT_PARAMS globals (read at call time, like the reference's module imports) + overrides."""
    p = {k: getattr(_P, k) for k in PARAM_NAMES}
    if overrides:
        unknown = set(overrides) - set(PARAM_NAMES)
        if unknown:
            raise KeyError(f"unknown INIT_PARAMS name(s): {sorted(unknown)}")
        p.update(overrides)
    return p


def cosmo_of(p: dict) -> cosmology.Cosmology:
    c = p["COSMO"]
    return c if isinstance(c, cosmology.Cosmology) else cosmology.Cosmology.from_dict(dict(c))


def ionize_setup(n, box_len, Z, p, *, fil, update, LE, scale=None, ref_compat=False):
    return schedule.ionize_setup(
        int(n), float(box_len), float(Z), zeta=float(p["ZETA"]), t_vir_min=float(p["ION_Tvir_MIN"]),
        R_max=float(p["R_BUBBLE_MAX"]), R_min=float(p["R_BUBBLE_MIN"]),
        delta_r_factor=float(p["DELTA_R_FACTOR"]), cosmo=cosmo_of(p), linear=bool(LE),
        filter_type=int(fil), update=int(update), ref_compat=ref_compat, scale=scale)


_plans: "collections.OrderedDict" = collections.OrderedDict()
_plans_lock = threading.Lock()
MAX_CACHED_PLANS = 8


def plan_for(n: int, box_len: float, max_radii: int, device, lane: int = 0):
    """A cached ExcursionSetPlan for (n, box_len, device) with room for max_radii radii; ``lane``
    selects one of several plans of the same size (boxes running side by side)."""
    from ..engine import ExcursionSetPlan
    import torch
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    key = (int(n), float(box_len), str(dev), int(lane))
    with _plans_lock:
        plan = _plans.get(key)
        if plan is not None and plan.max_radii >= max_radii:
            _plans.move_to_end(key)
            return plan
        if plan is not None:
            _plans.pop(key).close()
        plan = ExcursionSetPlan(n, box_len, max_radii=max(64, max_radii), device=dev)
        from ..autotune import ensure_tuned
        ensure_tuned(plan)
        _plans[key] = plan
        while len(_plans) > MAX_CACHED_PLANS:
            _plans.popitem(last=False)[1].close()
        return plan


def to_device(x, device):
    """(device float32 tensor, kind) for a numpy array or torch tensor input."""
    import torch
    if isinstance(x, torch.Tensor):
        kind = "torch-cuda" if x.is_cuda else "torch-cpu"
        t = x.to(device=device, dtype=torch.float32, non_blocking=True)
    else:
        kind = "numpy"
        a = np.ascontiguousarray(x, dtype=np.float32)
        t = torch.from_numpy(a).to(device, non_blocking=False)
    return t.contiguous(), kind


def to_host(t, kind, out=None):
    """Copy a device result back in the caller's container type (into out when given)."""
    import torch
    if kind == "torch-cuda":
        if out is not None:
            out.copy_(t)
            return out
        return t
    if out is not None:
        if isinstance(out, torch.Tensor):
            out.copy_(t, non_blocking=out.is_pinned())
            return out
        np.copyto(out, t.cpu().numpy())
        return out
    host = t.cpu()
    return host if kind == "torch-cpu" else host.numpy()
