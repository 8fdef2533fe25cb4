"""Density evolution on the GPU: the Zel'dovich mass move and the linear rescale that produce the
excursion-set input boxes (21cmpy's Programs/perturb_field.py:39-128, perturb_field.cu:90-132).

``PerturbPlan`` owns the device tables and the fixed-point accumulator of one (DIM, HII_DIM) pair;
its ``move_mass`` runs ``pf_move_mass`` (integer atomics, so the result does not depend on the
order in which the scattered masses land).  ``evolve_linear`` runs ``pf_evolve_linear``.
``updated_velocities`` recomputes the velocity boxes at the evolved redshift
(perturb_field.py:110-125) with the engine's real FFTs and the initial-conditions k-space kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream(device, stream=None):
    s = stream if stream is not None else torch.cuda.current_stream(device)
    return C.c_void_p(s.cuda_stream)


def _check_f32(t: torch.Tensor, shape, name, device):
    if not (isinstance(t, torch.Tensor) and t.dtype == torch.float32 and t.is_contiguous()
            and t.device == device and tuple(t.shape) == tuple(shape)):
        raise ValueError(f"{name}: need a contiguous float32 tensor of shape {tuple(shape)} on {device}")


class PerturbPlan:
    """Zel'dovich move of a DIM^3 initial-conditions box onto an HII_DIM^3 grid."""

    def __init__(self, dim: int, hii_dim: int, pixel_factor: float | None = None, device=None):
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.dim, self.hii_dim = int(dim), int(hii_dim)
        pf = np.float32(self.dim) / np.float32(self.hii_dim) if pixel_factor is None else np.float32(pixel_factor)
        self.pixel_factor = float(pf)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check("pf_plan_create", self.lib.pf_plan_create(self.dim, self.hii_dim, C.c_float(pf), C.byref(h)),
                       self.lib)
        self.handle = h

    def move_mass(self, delta, vx, vy, vz, init_growth: float, disp_scale: float, mass_factor: float,
                  out=None, stream=None) -> torch.Tensor:
        """updated [HII^3] = (sum of 1 + init_growth * delta over the cells landing in each HII cell)
        / mass_factor - 1, cells moved by v * disp_scale box lengths (perturb_field.py:91-101)."""
        d, s = (self.dim,) * 3, (self.hii_dim,) * 3
        _check_f32(delta, d, "delta", self.device)
        for name, v in (("vx", vx), ("vy", vy), ("vz", vz)):
            _check_f32(v, s, name, self.device)
        if out is None:
            out = torch.empty(s, dtype=torch.float32, device=self.device)
        _check_f32(out, s, "out", self.device)
        rc = self.lib.pf_move_mass(self.handle, _ptr(delta), _ptr(vx), _ptr(vy), _ptr(vz),
                                   C.c_float(float(np.float32(init_growth))), C.c_float(float(np.float32(disp_scale))),
                                   C.c_float(float(np.float32(mass_factor))), _ptr(out), _stream(self.device, stream))
        _lib.check("pf_move_mass", rc, self.lib)
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pf_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def evolve_linear(delta: torch.Tensor, growth: float, out=None, stream=None) -> torch.Tensor:
    """delta * growth in float32 on the device (perturb_field.py:43-47)."""
    lib = _lib.load()
    if not (isinstance(delta, torch.Tensor) and delta.is_cuda and delta.dtype == torch.float32 and delta.is_contiguous()):
        raise ValueError("delta: need a contiguous float32 CUDA tensor")
    if out is None:
        out = torch.empty_like(delta)
    _check_f32(out, delta.shape, "out", delta.device)
    rc = lib.pf_evolve_linear(delta.numel(), _ptr(delta), C.c_float(float(np.float32(growth))), _ptr(out),
                              _stream(delta.device, stream))
    _lib.check("pf_evolve_linear", rc, lib)
    return out


def updated_velocities(deltax: torch.Tensor, hii_dim: int, box_len: float, growth_rate: float,
                       pixel_factor: float | None = None, filter_type: int = 0, ref_compat: bool = False) -> dict:
    """Velocity boxes of the DIM^3 density ``deltax`` (perturb_field.py:110-125): per component c,
    (dD/dt / D) IFFT(W(kR) i k_c / k^2 FFT(deltax)) with a normalised inverse, R = L_FACTOR *
    BOX_LEN / HII_DIM, subsampled onto HII_DIM^3 (nearest cell).  Returns {"vx", "vy", "vz"}."""
    from .initial import InitialConditions
    dim = int(deltax.shape[0])
    _check_f32(deltax, (dim,) * 3, "deltax", deltax.device)
    with InitialConditions(dim, hii_dim, box_len, device=deltax.device) as ic:
        H = ic.plan.fft_r2c(deltax)
        scale = float(np.float32(growth_rate)) / float(dim) ** 3
        return ic.velocities(H, scale, filter_type, ref_compat, pixel_factor=pixel_factor)
