"""Initial conditions on the GPU: the Gaussian random density field at z = 0, its smoothed and
subsampled copy, and the Zel'dovich displacement (velocity / D-dot) boxes that perturb_field moves
the mass with (21cmpy's Programs/initialize.py:33-111, initialize.cu:58-95, 133-190).

Pipeline per box: normals -> ``ic_spectrum`` (sqrt(P V) per mode, P linearly interpolated in a
512-entry table as the reference does) -> the engine's inverse real FFT (``es_fft_c2r``) -> scale;
for the smoothed density and each displacement component, ``ic_shape`` (window W(kR) with
R = L_FACTOR * BOX_LEN / HII_DIM, times i k_c / k^2) -> inverse FFT -> ``ic_subsample`` (nearest
cell, scaled).  Normals come from a seeded torch generator on the device (the reference uses
PyCUDA's MRG32k3a); they can also be passed in.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib, cosmology

TABLE_N = 512                    # BLOCK_VOLUME entries of the P(k) table (initialize.py:21-26)
L_FACTOR = np.float32(0.620350491)


def pk_table(dim: int, box_len: float, cosmo: cosmology.Cosmology = cosmology.PLANCK13):
    """K log-spaced from DELTA_K / 10 to DELTA_K sqrt(3) DIM and P(K) at z = 0, float32
    (initialize.py:21-26)."""
    dk = float(np.float32(2 * np.pi / np.float32(box_len)))
    K = np.logspace(np.log10(dk / 10.0), np.log10(dk * np.sqrt(3.0) * dim), TABLE_N)
    P = cosmology.power_spectrum_z0(K, cosmo)
    return K.astype(np.float32), P.astype(np.float32)


def _p(t):
    return C.c_void_p(t.data_ptr())


class InitialConditions:
    """Initial-conditions boxes for a DIM^3 field of side box_len and its HII_DIM^3 copies."""

    def __init__(self, dim: int, hii_dim: int, box_len: float, cosmo=cosmology.PLANCK13, device=None):
        from .engine import ExcursionSetPlan
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.dim, self.hii_dim, self.box_len = int(dim), int(hii_dim), float(np.float32(box_len))
        self.cosmo = cosmo
        self.plan = ExcursionSetPlan(self.dim, self.box_len, max_radii=1, device=self.device)
        K, P = pk_table(self.dim, self.box_len, cosmo)
        self.K = torch.from_numpy(K).to(self.device)
        self.P = torch.from_numpy(P).to(self.device)
        self.pixel_factor = np.float32(self.dim) / np.float32(self.hii_dim)
        self.smooth_R = float(np.float32(L_FACTOR * np.float32(self.box_len) / np.float32(self.hii_dim)))
        # the unnormalised inverse FFT divided by the reference's IFFT normalisation and scale^3
        self.norm = float(1.0 / float(self.box_len) ** 3)

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def normals(self, seed: int):
        """Two [DIM][DIM][DIM/2+1] float32 normal arrays (real and imaginary parts)."""
        g = torch.Generator(device=self.device).manual_seed(int(seed))
        shape = (self.dim, self.dim, self.dim // 2 + 1)
        return (torch.randn(shape, generator=g, device=self.device), torch.randn(shape, generator=g, device=self.device))

    def spectrum(self, nre: torch.Tensor, nim: torch.Tensor) -> torch.Tensor:
        n = self.dim
        out = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=self.device)
        rc = self.lib.ic_spectrum(n, C.c_float(self.box_len), _p(nre.contiguous()), _p(nim.contiguous()),
                                  _p(self.K), _p(self.P), TABLE_N, _p(out), self._stream())
        _lib.check("ic_spectrum", rc, self.lib)
        return out

    def shaped(self, H: torch.Tensor, component: int, filter_type: int = 0, ref_compat: bool = False) -> torch.Tensor:
        out = torch.empty_like(H)
        rc = self.lib.ic_shape(self.dim, C.c_float(self.box_len), _p(H), int(component), int(filter_type),
                               C.c_float(self.smooth_R), int(ref_compat), _p(out), self._stream())
        _lib.check("ic_shape", rc, self.lib)
        return out

    def subsample(self, large: torch.Tensor, scale: float, size: int | None = None, pixel_factor=None) -> torch.Tensor:
        sw = self.hii_dim if size is None else int(size)
        pf = self.pixel_factor if pixel_factor is None else np.float32(pixel_factor)
        out = torch.empty((sw,) * 3, dtype=torch.float32, device=self.device)
        rc = self.lib.ic_subsample(self.dim, sw, C.c_float(float(pf)), C.c_float(float(np.float32(scale))),
                                   _p(large), _p(out), self._stream())
        _lib.check("ic_subsample", rc, self.lib)
        return out

    def generate(self, seed: int = 0, normals=None, filter_type: int = 0, ref_compat: bool = False) -> dict:
        """{"deltax": DIM^3 density at z = 0, "smoothed": HII_DIM^3 smoothed density,
        "vx", "vy", "vz": HII_DIM^3 displacement per unit growth (initialize.py:83-109)}."""
        nre, nim = self.normals(seed) if normals is None else normals
        H = self.spectrum(nre, nim)
        out = {"spectrum": H}
        full = self.plan.fft_c2r(H)
        out["deltax"] = self.subsample(full, self.norm, size=self.dim, pixel_factor=1.0)
        del full
        S = self.plan.fft_c2r(self.shaped(H, -1, filter_type, ref_compat))
        out["smoothed"] = self.subsample(S, self.norm)
        del S
        out.update(self.velocities(H, self.norm, filter_type, ref_compat))
        return out

    def velocities(self, H: torch.Tensor, scale: float, filter_type: int = 0, ref_compat: bool = False,
                   pixel_factor=None) -> dict:
        """{"vx", "vy", "vz"}: scale * IFFT(W(kR) i k_c / k^2 H) subsampled onto HII_DIM^3, the
        inverse FFT unnormalised (set_velocity, HII_filter and subsample: initialize.cu:12-40,
        133-190; perturb_field.cu:39-88)."""
        out = {}
        for c, name in enumerate(("vx", "vy", "vz")):
            V = self.plan.fft_c2r(self.shaped(H, c, filter_type, ref_compat))
            out[name] = self.subsample(V, scale, pixel_factor=pixel_factor)
            del V
        return out

    def close(self):
        if getattr(self, "plan", None) is not None:
            self.plan.close()
            self.plan = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
