"""Host-side set-up of one excursion-set run: the descending radius schedule and its scalars.

This is the FP64 host half of ``conv_bubbles`` (Programs/find_HII_bubbles.py:54-60, 83-92,
113-128, 189).  The GPU receives only the float32 values computed here, exactly the scalars the
reference passes to its kernels (R, denom, DELTAC, ZETA, fc_mean_ps), so the CUDA path and the
oracle consume identical inputs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .cosmology import Cosmology, SigmaTable, collapse_fraction, sig_del, sigma_table

# Parameter_files/INIT_PARAMS.py:31 -- (4 pi / 3)^(-1/3), cube side to filter radius
L_FACTOR = float(np.float32(0.620350491))


class ExcursionSetError(Exception):
    """Raised where the reference raises a bare ``Exception`` (find_HII_bubbles.py:116-118)."""


@dataclass
class RadiusStep:
    R: np.float32          # filter radius [Mpc] (float32, as the reference's ``R = np.float32(R)``)
    sigma2: np.float32     # sigma^2(R) at z = 0 (``S0 = np.float32(sig0(R))``)
    denom: np.float32      # sqrt(2 (sigma_min^2 - sigma^2(R))) as float32
    final: bool            # last radius: paint partial ionisations (final_kernel)


@dataclass
class IonizeSetup:
    """All scalars of one box's excursion-set run (what ``conv_bubbles`` derives on the host)."""
    n: int
    box_len: float
    z: float
    zeta: float
    t_vir_min: float
    sigma_min: float
    delta_c: float
    fc_mean_ps: np.float32
    growth_scale: np.float32       # multiply the density by this before filtering
    normalize_mean: bool           # reference LE=False: rescale fcoll by fc_mean_ps / <fcoll>
    steps: list = field(default_factory=list)
    filter_type: int = 0
    update: int = 0
    ref_compat: bool = False

    @property
    def scale(self) -> float:
        return self.box_len / self.n

    @property
    def n_radii(self) -> int:
        return len(self.steps)

    def radii(self) -> np.ndarray:
        return np.array([s.R for s in self.steps], dtype=np.float32)

    def denoms(self) -> np.ndarray:
        return np.array([s.denom for s in self.steps], dtype=np.float32)

    @property
    def deltac32(self) -> np.float32:
        # the reference pastes repr(deltac) into ``float deltac = ...`` (find_bubbles.cu:54)
        return np.float32(self.delta_c)


def radius_schedule(R_max: float, R_min: float, delta_r_factor: float, scale: float,
                    smin: float, sig2) -> list:
    """Descending radii R_max, R_max/f, ... as in find_HII_bubbles.py:92, 113-128, 189.

    The loop stops after the radius whose successor R/f is below the cell scale
    L_FACTOR * scale or below R_min.  As in the reference, R is rounded to float32 at every
    step and the successor is computed in double precision from that float32 value.
    """
    if not (R_max > 0 and delta_r_factor > 1.0 and scale > 0):
        raise ExcursionSetError("radius schedule needs R_max > 0, DELTA_R_FACTOR > 1, scale > 0")
    cell = L_FACTOR * scale
    if R_min < cell and 2.0 * (smin - sig2(cell)) < 0.0:
        # find_HII_bubbles.py:114-118: sigma^2 at the cell scale exceeds sigma_min^2
        raise ExcursionSetError("sigma^2(L_FACTOR*scale) exceeds sigma_min^2: cells finer than "
                                "the minimum halo scale")
    steps = []
    R = float(R_max)
    while True:
        final = (R / delta_r_factor) <= cell or (R / delta_r_factor) <= R_min
        R32 = np.float32(R)
        S0 = np.float32(sig2(float(R32)))
        arg = 2.0 * (smin - float(S0))
        if arg <= 0.0:
            raise ExcursionSetError(f"sigma^2(R={float(R32)}) >= sigma_min^2: R below the minimum "
                                    "halo scale")
        steps.append(RadiusStep(R32, S0, np.float32(math.sqrt(arg)), final))
        if final:
            return steps
        if len(steps) > 4096:
            raise ExcursionSetError("radius schedule does not terminate")
        R = float(R32) / delta_r_factor


def ionize_setup(n: int, box_len: float, z: float, *, zeta: float, t_vir_min: float,
                 R_max: float, R_min: float = 0.5, delta_r_factor: float = 1.1,
                 cosmo: Cosmology, linear: bool = False, filter_type: int = 0, update: int = 0,
                 ref_compat: bool = False, scale: float | None = None,
                 table: SigmaTable | None = None) -> IonizeSetup:
    """Everything ``conv_bubbles`` computes on the host before its radius loop.

    ``linear=True`` is the reference's ``LE=True`` (density already linear at z = 0: no growth
    rescale and no mean normalisation, find_HII_bubbles.py:83-85, 158-160); ``linear=False`` is
    the ``updated_*`` density at redshift z.
    """
    if n <= 0 or n % 2:
        raise ExcursionSetError(f"HII_DIM must be a positive even integer, got {n}")
    if box_len <= 0:
        raise ExcursionSetError("BOX_LEN must be positive")
    if zeta <= 0:
        raise ExcursionSetError("ZETA must be positive")
    table = table or sigma_table(cosmo)
    sigma_min, delta_c = sig_del(t_vir_min, z, cosmo, table)
    smin = sigma_min ** 2
    fc_mean = np.float32(collapse_fraction(sigma_min, delta_c))
    scale = box_len / n if scale is None else float(scale)
    steps = radius_schedule(R_max, R_min, delta_r_factor, scale, smin, table.sigma2)
    growth = np.float32(delta_c / 1.686)     # find_HII_bubbles.py:58 (= 1/D(z))
    return IonizeSetup(n=n, box_len=float(box_len), z=float(z), zeta=float(zeta),
                       t_vir_min=float(t_vir_min), sigma_min=sigma_min, delta_c=delta_c,
                       fc_mean_ps=fc_mean,
                       growth_scale=np.float32(1.0) if linear else growth,
                       normalize_mean=not linear, steps=steps, filter_type=int(filter_type),
                       update=int(update), ref_compat=bool(ref_compat))


def delta_k(box_len: float) -> np.float32:
    """DELTA_K = float32(2 pi / BOX_LEN) with BOX_LEN rounded to float32 (delta_T.py:51-52)."""
    return np.float32(2.0 * math.pi / float(np.float32(box_len)))


def pk_edges(n: int, box_len: float, num_bins: int, edge_dim: int | None = None) -> np.ndarray:
    """Bin edges K = logspace(log10 dk, log10(dk sqrt(3) DIM), NUM_BINS) as float32 (delta_T.py:87).

    The reference uses the large-box DIM for the top edge; by default the box's own HII_DIM is
    used (``edge_dim`` restores the reference's choice).
    """
    dk = float(delta_k(box_len))
    top = edge_dim if edge_dim is not None else n
    return np.float32(np.logspace(np.log10(dk), np.log10(dk * np.sqrt(3.0) * top), num_bins))


def pk_k2_thresholds(n: int, box_len: float, edges: np.ndarray) -> np.ndarray:
    """Integer thresholds T[b] = max{m : dk sqrt(m) <= K[b]} (int32; -1 when none).

    A mode with integer |k/dk|^2 = m falls in the first bin b with K[b] >= |k| (delta_T.cu:25-26),
    i.e. the first b with m <= T[b].  Deciding the comparison once, in float64 on the host,
    makes the bin of every mode identical on the GPU and in the oracle.
    """
    dk = float(delta_k(box_len))
    kmax2 = 3 * (n // 2) ** 2
    out = np.empty(len(edges), dtype=np.int64)
    for b, e in enumerate(np.asarray(edges, dtype=np.float64)):
        m = int(math.floor((e / dk) ** 2)) + 2
        while m >= 0 and dk * math.sqrt(m) > e:
            m -= 1
        out[b] = min(m, kmax2)
    return out.astype(np.int32)
