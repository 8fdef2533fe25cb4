"""Batched form of the engine: many boxes of uneven HII_DIM and parameters in one persistent
launch, replayed from a captured CUDA graph (no counterpart in the reference, which runs one box
per ``conv_bubbles`` call).

Each box is a (device density, :class:`~.schedule.IonizeSetup`) pair; outputs are x_HI boxes and
the mean x_HI of every box.  The persistent kernel walks a work queue of (box, pass, tile) items:
boxes are dealt to lanes balanced by N^3 * N_R and the lanes advance side by side, so small boxes
keep the whole GPU busy while only a few boxes' workspaces are live at a time.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .schedule import IonizeSetup, pk_k2_thresholds


def _params(st: IonizeSetup, output: int):
    rad = (_lib.es_radius * st.n_radii)()
    for i, s in enumerate(st.steps):
        rad[i].R = float(s.R)
        rad[i].denom = float(s.denom)
    prm = _lib.es_ionize_params(
        n_radii=st.n_radii, radii=rad, delta_c=float(st.deltac32), fc_mean_ps=float(st.fc_mean_ps),
        zeta=float(np.float32(st.zeta)), growth_scale=float(st.growth_scale),
        normalize_mean=int(st.normalize_mean), filter_type=int(st.filter_type), update=int(st.update),
        ref_compat=int(st.ref_compat), output=output)
    return prm, rad


class BatchedExcursionSet:
    """x_HI of many boxes in one persistent launch (``es_batch_*``).

    ``t_factors`` (one brightness-temperature factor per box, see
    ``cosmology.brightness_temperature_factor``) adds delta_T and its mean to every box's outputs,
    and ``pk_edges`` (one array of bin edges in 1/Mpc per box, or one for all) its binned P(k)
    (delta_T.py:73-98), all inside the same launch: ``self.dT``, ``self.ave`` and ``self.pk``
    ((3, nbins) per box: ps_ave, k_ave, count)."""

    def __init__(self, boxes, output: str = "xH", use_graph: bool = True, device=None, lanes: int = None,
                 chunk: int = None, t_factors=None, pk_edges=None, dimensional: bool = False):
        if not torch.cuda.is_available():
            raise _lib.EngineUnavailable("the batched engine needs a CUDA device")
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.use_graph = bool(use_graph)
        self.inputs, self.setups = [], []
        for d, st in boxes:
            if not isinstance(d, torch.Tensor) or d.device != self.device or d.dtype != torch.float32:
                raise ValueError("densities must be float32 tensors on the batch's device")
            n = st.n
            if tuple(d.shape) != (n, n, n) or not d.is_contiguous():
                raise ValueError(f"density of a {n}^3 box must be a contiguous ({n}, {n}, {n}) tensor")
            self.inputs.append(d)
            self.setups.append(st)
        cnt = len(self.setups)
        if cnt == 0:
            raise ValueError("empty batch")
        self.out = [torch.empty_like(d) for d in self.inputs]
        self.nf = torch.zeros(cnt, dtype=torch.float32, device=self.device)
        self.dT = self.ave = self.pk = None
        if pk_edges is not None and t_factors is None:
            raise ValueError("P(k) is of delta_T: give t_factors too")
        if t_factors is not None:
            if len(t_factors) != cnt:
                raise ValueError("one brightness-temperature factor per box")
            self.dT = [torch.empty_like(d) for d in self.inputs]
            self.ave = torch.zeros(cnt, dtype=torch.float32, device=self.device)
        thr = [None] * cnt
        if pk_edges is not None:
            edges = [pk_edges] * cnt if np.ndim(pk_edges[0]) == 0 else list(pk_edges)
            if len(edges) != cnt:
                raise ValueError("one array of P(k) bin edges per box (or one for all)")
            thr = [pk_k2_thresholds(st.n, st.box_len, np.asarray(e)) for st, e in zip(self.setups, edges)]
            self.pk = [torch.zeros((3, len(t)), dtype=torch.float32, device=self.device) for t in thr]
        arr = (_lib.es_batch_box * cnt)()
        keep = []
        for i, (d, st) in enumerate(zip(self.inputs, self.setups)):
            prm, rad = _params(st, 0 if output == "xH" else 1)
            keep.append(rad)
            arr[i].n = st.n
            arr[i].box_len = st.box_len
            arr[i].delta = C.c_void_p(d.data_ptr())
            arr[i].out = C.c_void_p(self.out[i].data_ptr())
            arr[i].nf = C.c_void_p(self.nf.data_ptr() + 4 * i)
            arr[i].params = prm
            if self.dT is not None:
                arr[i].t_factor = float(t_factors[i])
                arr[i].dT = C.c_void_p(self.dT[i].data_ptr())
                arr[i].ave = C.c_void_p(self.ave.data_ptr() + 4 * i)
            if thr[i] is not None:
                cthr = (C.c_int * len(thr[i]))(*[int(v) for v in thr[i]])
                keep.append(cthr)
                arr[i].k2_thresholds = cthr
                arr[i].nbins = len(thr[i])
                arr[i].dimensional = int(dimensional)
                arr[i].pk = C.c_void_p(self.pk[i].data_ptr())
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.es_batch_create(arr, cnt, C.byref(h))
        _lib.check("es_batch_create", rc, self.lib)
        self._h = h
        if lanes is not None or chunk is not None:
            self.set_schedule(0 if lanes is None else lanes, 1 if chunk is None else chunk)

    def set_schedule(self, lanes: int, chunk: int):
        """``lanes`` boxes in flight (0: every box its own lane), ``chunk`` tiles per ticket."""
        _lib.check("es_batch_set_schedule", self.lib.es_batch_set_schedule(self.handle, int(lanes), int(chunk)),
                   self.lib)

    def profile(self, enable: bool = True):
        """Clear and enable (or disable) the per-op cycle counters of the persistent launch."""
        _lib.check("es_batch_profile", self.lib.es_batch_profile(self.handle, int(enable)), self.lib)

    def profile_read(self) -> dict:
        """Per op: SM clock cycles CTAs spent in its tiles, tiles, cycles finding and awaiting its
        tickets, tickets (summed over the launches since ``profile(True)``)."""
        buf = (C.c_ulonglong * (4 * len(OPS)))()
        _lib.check("es_batch_profile_read", self.lib.es_batch_profile_read(self.handle, buf, len(OPS)), self.lib)
        out = {}
        for i, name in enumerate(OPS):
            cyc, tiles, wait, tickets = (int(buf[4 * i + k]) for k in range(4))
            if tiles:
                out[name] = {"tile_cycles": cyc, "tiles": tiles, "wait_cycles": wait, "tickets": tickets}
        return out

    def schedule(self) -> dict:
        lanes, chunk, tickets = C.c_int(), C.c_int(), C.c_uint()
        _lib.check("es_batch_get_schedule", self.lib.es_batch_get_schedule(
            self.handle, C.byref(lanes), C.byref(chunk), C.byref(tickets)), self.lib)
        return {"lanes": lanes.value, "chunk": chunk.value, "tickets": tickets.value}

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("batch is closed")
        return self._h

    def run(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            rc = self.lib.es_batch_run(self.handle, int(self.use_graph), C.c_void_p(s.cuda_stream))
        _lib.check("es_batch_run", rc, self.lib)
        return self.out, self.nf

    def check(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check("es_batch_check", self.lib.es_batch_check(self.handle, C.c_void_p(s.cuda_stream)), self.lib)

    def info(self) -> dict:
        g, p, sm = C.c_int(), C.c_int(), C.c_int()
        t = C.c_uint()
        _lib.check("es_batch_info", self.lib.es_batch_info(self.handle, C.byref(g), C.byref(p), C.byref(t), C.byref(sm)), self.lib)
        return {"grid": g.value, "passes": p.value, "tiles": t.value, "smem": sm.value, **self.schedule()}

    def voxel_radius_updates(self) -> int:
        return sum(st.n ** 3 * st.n_radii for st in self.setups)

    def close(self):
        if getattr(self, "_h", None) is not None:
            self.lib.es_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class PlanGraphBatch:
    """x_HI of many boxes through per-box plans on concurrent streams, captured once into a CUDA
    graph and replayed.

    Boxes are grouped by (HII_DIM, BOX_LEN); each group gets up to ``lanes`` plans, each with its own
    stream, and a lane runs its boxes (forward transform, radius loop, final step) one after the
    other while the lanes of all groups run side by side.  The plans use the TMA passes, whose
    radius parameters are kernel arguments, so a whole batch is a static graph; ``tune`` applies
    the autotuner's configuration of every box size (overlapped radii included).
    """

    def __init__(self, boxes, output: str = "xH", lanes: int = 2, use_graph: bool = True, tune: bool = True,
                 device=None):
        from .autotune import ensure_tuned
        from .engine import ExcursionSetPlan
        if not torch.cuda.is_available():
            raise _lib.EngineUnavailable("the batched engine needs a CUDA device")
        if lanes < 1:
            raise ValueError("lanes must be >= 1")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.output = output
        self.inputs, self.setups = [], []
        for d, st in boxes:
            if not isinstance(d, torch.Tensor) or d.device != self.device or d.dtype != torch.float32:
                raise ValueError("densities must be float32 tensors on the batch's device")
            self.inputs.append(d)
            self.setups.append(st)
        if not self.setups:
            raise ValueError("empty batch")
        self.out = [torch.empty_like(d) for d in self.inputs]
        self.nf = torch.zeros(len(self.setups), dtype=torch.float32, device=self.device)
        groups: dict = {}
        for i, st in enumerate(self.setups):
            groups.setdefault((st.n, float(st.box_len)), []).append(i)
        self.lanes = []                       # (plan, stream, [box indices])
        with torch.cuda.device(self.device):
            for (n, L), idx in sorted(groups.items()):
                k = min(lanes, len(idx))
                radii = max(self.setups[i].n_radii for i in idx)
                for j in range(k):
                    plan = ExcursionSetPlan(n, L, max_radii=max(64, radii), device=self.device)
                    if tune:
                        ensure_tuned(plan)
                    if plan.col_variant != 1:
                        plan.col_variant = 1           # graph capture needs the TMA passes
                    self.lanes.append((plan, torch.cuda.Stream(self.device), idx[j::k]))
        self.use_graph = bool(use_graph)
        self.graph = None

    def _body(self):
        cur = torch.cuda.current_stream(self.device)
        fork = torch.cuda.Event()
        fork.record(cur)
        for _plan, s, _idx in self.lanes:
            s.wait_event(fork)
        longest = max(len(idx) for _p, _s, idx in self.lanes)
        for step in range(longest):                    # hand every lane its next box in turn
            for plan, s, idx in self.lanes:
                if step < len(idx):
                    i = idx[step]
                    plan.run(self.inputs[i], self.setups[i], out=self.out[i], nf=self.nf[i:i + 1],
                             output=self.output, stream=s)
        for _plan, s, _idx in self.lanes:
            cur.wait_stream(s)

    def run(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device), torch.cuda.stream(s):
            if not self.use_graph:
                self._body()
            else:
                if self.graph is None:
                    self._body()                       # warm-up outside the capture
                    torch.cuda.synchronize(self.device)
                    self.graph = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(self.graph):
                        self._body()
                self.graph.replay()
        return self.out, self.nf

    def check(self, stream=None):
        for plan, _s, _idx in self.lanes:
            plan.check(stream)

    def voxel_radius_updates(self) -> int:
        return sum(st.n ** 3 * st.n_radii for st in self.setups)

    def info(self) -> dict:
        return {"lanes": len(self.lanes), "boxes": len(self.setups),
                "plans": sorted({(p.n, len(idx)) for p, _s, idx in self.lanes})}

    def close(self):
        self.graph = None
        for plan, _s, _idx in getattr(self, "lanes", []):
            plan.close()
        self.lanes = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


OPS = ("row_r2c", "y_fwd", "z_fwd", "z_inv", "y_inv", "row_c2r", "final", "wtab", "paint", "pk_r2c", "z_fwd_pk")


def queue_plan(ns, n_radii, lanes: int = 0, chunk: int = 1, update=None, pk=None):
    """The persistent launch's work queue for boxes of HII_DIM ``ns`` with ``n_radii`` radii (update
    modes ``update`` and P(k) flags ``pk``, default all 0) under a schedule, built on the host by
    ``es_batch_queue`` (no device needed): a list of {box, op, radius, tiles, first, tickets, dep,
    dep2} in queue order."""
    lib = _lib.load()
    cnt = len(ns)
    upd = [0] * cnt if update is None else [int(u) for u in update]
    pks = [0] * cnt if pk is None else [int(u) for u in pk]
    n_arr = (C.c_int * cnt)(*[int(v) for v in ns])
    r_arr = (C.c_int * cnt)(*[int(v) for v in n_radii])
    u_arr = (C.c_int * cnt)(*upd)
    k_arr = (C.c_int * cnt)(*pks)
    cap = sum(5 + 3 * int(r) + (int(r) - 1 if u else 0) + 3 * k for r, u, k in zip(n_radii, upd, pks))
    out = (C.c_int * (8 * cap))()
    rc = lib.es_batch_queue(n_arr, r_arr, u_arr, k_arr, cnt, int(lanes), int(chunk), out, cap)
    _lib.check("es_batch_queue", min(rc, 0), lib)
    keys = ("box", "op", "radius", "tiles", "first", "tickets", "dep", "dep2")
    q = [dict(zip(keys, out[8 * k:8 * k + 8])) for k in range(rc)]
    for d in q:
        d["op"] = OPS[d["op"]]
    return q


def boxes_from_specs(specs, device=None, cosmo=None, table=None):
    """(device density, IonizeSetup) pairs for BoxSpec entries (seeded GRF at each box's z)."""
    from .cosmology import BASELINE_COSMO
    from .grf import density_box
    from .schedule import ionize_setup
    cosmo = cosmo or BASELINE_COSMO
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = []
    for s in specs:
        d = torch.from_numpy(density_box(s.n, s.box_len, s.seed, s.z, cosmo)).to(dev)
        st = ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min, R_max=s.R_max,
                          cosmo=cosmo)
        out.append((d, st))
    return out


def box_cost(n: int, n_radii: int) -> int:
    """Work of one box: N^3 voxels times its number of filter radii (each radius is one inverse
    transform with the fcoll epilogue; the forward transform and the final step are per box)."""
    return int(n) ** 3 * int(n_radii)


def shard_specs(specs, world: int, cosmo=None):
    """Splits BoxSpec work items over ranks by their cost N^3 * N_R (longest processing time first).

    The radius count of every box comes from its own schedule (R_mfp, cell size), so boxes of the
    same size with different R_mfp weigh differently.  Returns one list of spec indices per rank.
    """
    from .cosmology import BASELINE_COSMO
    from .schedule import ionize_setup
    cosmo = cosmo or BASELINE_COSMO
    costs = [box_cost(s.n, ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min,
                                        R_max=s.R_max, cosmo=cosmo).n_radii) for s in specs]
    return shard(costs, world)


def shard(costs, world: int):
    """Longest-processing-time split of work items (cost per item) over `world` ranks.

    Returns one list of item indices per rank; every item appears exactly once.  Boxes are
    independent, so ranks need no collective on the data path.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += costs[i]
    return [sorted(p) for p in parts]
