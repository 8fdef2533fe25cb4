"""Seeded Gaussian random density fields and the synthetic benchmark workloads.

The reference's own initial conditions (Programs/initialize.py:33-111) draw a k-space field on
the GPU; the benchmark boxes here are instead drawn on the host from a seeded
``numpy.random.Generator(PCG64(seed))``: real-space white noise -> rfftn -> multiply by
sqrt(P(k) N^3 / V) -> irfftn, then scaled by the linear growth D(z).  The files are named like
``perturb_field`` output (``updated_smoothed_deltax_z{z:06.2f}_{N}_{L}Mpc.npy``) so the
``LE=False`` branch of find_HII_bubbles.py:214-221 applies.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .cosmology import BASELINE_COSMO, Cosmology, growth_factor, power_spectrum_z0


def grf_z0(n: int, box_len: float, seed: int, cosmo: Cosmology = BASELINE_COSMO) -> np.ndarray:
    """Linear density contrast at z = 0 on an n^3 grid of side box_len [Mpc] (float64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    dk = 2.0 * math.pi / box_len
    kz = np.fft.fftfreq(n, d=1.0 / n) * dk
    kx = np.fft.rfftfreq(n, d=1.0 / n) * dk
    kmag = np.sqrt(kz[:, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2)
    amp = np.zeros_like(kmag)
    nz = kmag > 0
    amp[nz] = np.sqrt(power_spectrum_z0(kmag[nz], cosmo) * n ** 3 / box_len ** 3)
    wk *= amp
    return np.fft.irfftn(wk, s=(n, n, n), axes=(0, 1, 2))


def density_box(n: int, box_len: float, seed: int, z: float, cosmo: Cosmology = BASELINE_COSMO,
                base: np.ndarray | None = None) -> np.ndarray:
    """float32 density at redshift z: D(z) times the seeded z = 0 field."""
    d0 = grf_z0(n, box_len, seed, cosmo) if base is None else base
    return (d0 * growth_factor(z, cosmo)).astype(np.float32)


def density_filename(n: int, box_len: float, z: float) -> str:
    return f"updated_smoothed_deltax_z{z:06.2f}_{n}_{int(round(box_len))}Mpc.npy"


@dataclass
class BoxSpec:
    """One excursion-set unit of work: a density realisation plus its parameter point."""
    n: int
    box_len: float
    seed: int
    z: float
    zeta: float
    R_max: float
    t_vir_min: float


def sweep_256(seeds=range(4)) -> list:
    """HII_DIM=256, L=300 Mpc, seeds 0-3 x z = 6.0, 6.5, ..., 12.0; zeta=30, R_mfp=15, Tvir=1e4.

    ``seeds`` widens the sweep to more realisations of the same redshift grid (weak scaling over
    several GPUs: 4 seeds per GPU)."""
    zs = [6.0 + 0.5 * i for i in range(13)]
    return [BoxSpec(256, 300.0, s, z, 30.0, 15.0, 1.0e4) for s in seeds for z in zs]


def single_64() -> BoxSpec:
    """HII_DIM=64, L=100 Mpc, seed 0, z=8, zeta=30, R_mfp=15, Tvir=1e4 (CPU-runnable case)."""
    return BoxSpec(64, 100.0, 0, 8.0, 30.0, 15.0, 1.0e4)


def single_512() -> BoxSpec:
    """HII_DIM=512, L=600 Mpc, z=7.5, zeta=40, R_mfp=30 Mpc, Tvir=1e4."""
    return BoxSpec(512, 600.0, 0, 7.5, 40.0, 30.0, 1.0e4)


def uneven_batch(count: int = 64, first_seed: int = 100, dims=(64, 96, 128, 160),
                 param_seed: int = 12345) -> list:
    """Batched sweep: HII_DIM ~ U{64,96,128,160}, L = 1.5 N Mpc, seeds 100.., zeta ~ U[10,80],
    R_mfp ~ U[5,50] Mpc, log10 Tvir ~ U[4,5.3], z ~ U[6,10] (drawn from a fixed PCG64 stream)."""
    rng = np.random.Generator(np.random.PCG64(param_seed))
    out = []
    for i in range(count):
        n = int(rng.choice(dims))
        out.append(BoxSpec(n, 1.5 * n, first_seed + i, float(rng.uniform(6.0, 10.0)),
                           float(rng.uniform(10.0, 80.0)), float(rng.uniform(5.0, 50.0)),
                           float(10 ** rng.uniform(4.0, 5.3))))
    return out
