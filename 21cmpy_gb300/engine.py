"""Host side of the GB300 excursion-set engine: plans over the C ABI with torch device tensors.

:class:`ExcursionSetPlan` mirrors the per-box state ``conv_bubbles`` builds
(Programs/find_HII_bubbles.py:76-91: pyfft plan, device boxes) and exposes the three stages of
the reference path:

* :meth:`ExcursionSetPlan.ionize` -- the radius loop of ``conv_bubbles`` (l.121-192);
* :meth:`ExcursionSetPlan.delta_T` -- the brightness-temperature box of ``delta_T.run``
  (Programs/delta_T.py:73-76);
* :meth:`ExcursionSetPlan.power_spectrum` -- its binned power spectrum (delta_T.py:80-98).

All of them run on the CUDA engine; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .schedule import IonizeSetup, pk_k2_thresholds


def _stream_handle(device: torch.device, stream) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream(device)
    return C.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def supported_sizes() -> list:
    lib = _lib.load()
    buf = (C.c_int * 64)()
    n = lib.es_supported_sizes(buf, 64)
    return [buf[i] for i in range(min(n, 64))]


class ExcursionSetPlan:
    """Workspace and kernels for boxes of HII_DIM=n, BOX_LEN=box_len on one CUDA device."""

    def __init__(self, n: int, box_len: float, max_radii: int = 64, device=None):
        if not torch.cuda.is_available():
            raise _lib.EngineUnavailable("the excursion-set engine needs a CUDA device")
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise ValueError("plans live on a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.n = int(n)
        self.box_len = float(box_len)
        self.max_radii = int(max_radii)
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.es_plan_create(self.n, self.box_len, self.max_radii, C.byref(handle))
        _lib.check("es_plan_create", rc, self.lib)
        self._h = handle
        self._scalars = torch.zeros(4, dtype=torch.float32, device=self.device)

    # ------------------------------------------------------------------ helpers
    def _check_box(self, t: torch.Tensor, name: str):
        n = self.n
        if not isinstance(t, torch.Tensor) or t.device != self.device or t.dtype != torch.float32:
            raise ValueError(f"{name} must be a float32 tensor on {self.device}")
        if tuple(t.shape) != (n, n, n) or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous ({n}, {n}, {n}) box, got {tuple(t.shape)}")

    def _box(self, out, name):
        if out is None:
            return torch.empty((self.n,) * 3, dtype=torch.float32, device=self.device)
        self._check_box(out, name)
        return out

    def _scalar(self, t, idx):
        if t is None:
            return torch.empty(1, dtype=torch.float32, device=self.device)
        if t.device != self.device or t.dtype != torch.float32 or t.numel() < 1:
            raise ValueError("scalar outputs must be float32 device tensors")
        return t

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("plan is closed")
        return self._h

    def workspace_bytes(self) -> int:
        return int(self.lib.es_plan_workspace_bytes(self.n, self.max_radii))

    # ------------------------------------------------------------------ stages
    def forward(self, delta: torch.Tensor, stream=None):
        """Transform the density box once (the reference re-transforms per radius, l.141-144)."""
        self._check_box(delta, "delta")
        _lib.check("es_forward", self.lib.es_forward(self.handle, _ptr(delta), _stream_handle(self.device, stream)), self.lib)

    def ionize(self, setup: IonizeSetup, out: torch.Tensor | None = None, nf: torch.Tensor | None = None,
               output: str = "xH", stream=None):
        """Radius loop on the last forward()ed box; returns (out box, device nf = <x_HI>)."""
        if setup.n != self.n or abs(setup.box_len - self.box_len) > 1e-9 * self.box_len:
            raise ValueError("setup was made for a different box")
        if setup.n_radii > self.max_radii:
            raise ValueError(f"{setup.n_radii} radii exceed the plan's max_radii={self.max_radii}")
        out = self._box(out, "out")
        nf = self._scalar(nf, 0)
        rad = (_lib.es_radius * setup.n_radii)()
        for i, st in enumerate(setup.steps):
            rad[i].R = float(st.R)
            rad[i].denom = float(st.denom)
        prm = _lib.es_ionize_params(
            n_radii=setup.n_radii, radii=rad, delta_c=float(setup.deltac32),
            fc_mean_ps=float(setup.fc_mean_ps), zeta=float(np.float32(setup.zeta)),
            growth_scale=float(setup.growth_scale), normalize_mean=int(setup.normalize_mean),
            filter_type=int(setup.filter_type), update=int(setup.update),
            ref_compat=int(setup.ref_compat), output=0 if output == "xH" else 1)
        rc = self.lib.es_ionize(self.handle, C.byref(prm), _ptr(out), _ptr(nf), _stream_handle(self.device, stream))
        _lib.check("es_ionize", rc, self.lib)
        return out, nf

    def run(self, delta: torch.Tensor, setup: IonizeSetup, out=None, nf=None, output="xH", stream=None):
        self.forward(delta, stream)
        return self.ionize(setup, out, nf, output, stream)

    def delta_T(self, xH: torch.Tensor, delta: torch.Tensor, const_factor: float, out=None, ave=None, stream=None):
        """delta_T = const * x_HI * (1 + delta) and its device mean (delta_T.py:73-76)."""
        self._check_box(xH, "xH")
        self._check_box(delta, "delta")
        out = self._box(out, "dT")
        ave = self._scalar(ave, 1)
        rc = self.lib.es_delta_T(self.handle, _ptr(xH), _ptr(delta), C.c_float(float(np.float32(const_factor))),
                                 _ptr(out), _ptr(ave), _stream_handle(self.device, stream))
        _lib.check("es_delta_T", rc, self.lib)
        return out, ave

    def power_spectrum(self, dT: torch.Tensor, ave: torch.Tensor, edges, dimensional: bool = False,
                       out=None, stream=None):
        """Binned Delta^2(k) of (dT/ave - 1) V/N^3; returns a device (3, nbins) tensor of
        (ps_ave, k_ave, count) per bin (delta_T.py:87-98)."""
        self._check_box(dT, "dT")
        thr = pk_k2_thresholds(self.n, self.box_len, np.asarray(edges))
        nb = len(thr)
        if out is None:
            out = torch.empty((3, nb), dtype=torch.float32, device=self.device)
        cthr = (C.c_int * nb)(*[int(v) for v in thr])
        rc = self.lib.es_power_spectrum(self.handle, _ptr(dT), _ptr(ave), cthr, nb, int(dimensional),
                                        _ptr(out), _stream_handle(self.device, stream))
        _lib.check("es_power_spectrum", rc, self.lib)
        return out

    def fft_r2c(self, x: torch.Tensor, stream=None) -> torch.Tensor:
        """Unnormalised 3-D real FFT in numpy's rfftn layout (testing the transform passes)."""
        self._check_box(x, "x")
        out = torch.empty((self.n, self.n, self.n // 2 + 1), dtype=torch.complex64, device=self.device)
        _lib.check("es_fft_r2c", self.lib.es_fft_r2c(self.handle, _ptr(x), _ptr(out), _stream_handle(self.device, stream)), self.lib)
        return out

    def fft_c2r(self, X: torch.Tensor, stream=None) -> torch.Tensor:
        """Unnormalised inverse (numpy irfftn times n^3) from numpy's rfftn layout."""
        n = self.n
        if X.dtype != torch.complex64 or tuple(X.shape) != (n, n, n // 2 + 1) or X.device != self.device:
            raise ValueError("X must be a complex64 (n, n, n/2+1) device tensor")
        X = X.contiguous()
        out = torch.empty((n, n, n), dtype=torch.float32, device=self.device)
        _lib.check("es_fft_c2r", self.lib.es_fft_c2r(self.handle, _ptr(X), _ptr(out), _stream_handle(self.device, stream)), self.lib)
        return out

    # ------------------------------------------------------------------ options and health
    def set_option(self, option: int, value: int):
        _lib.check("es_plan_set_option", self.lib.es_plan_set_option(self.handle, int(option), int(value)), self.lib)

    def get_option(self, option: int) -> int:
        v = C.c_int()
        _lib.check("es_plan_get_option", self.lib.es_plan_get_option(self.handle, int(option), C.byref(v)), self.lib)
        return int(v.value)

    @property
    def col_variant(self) -> int:
        """Column-pass implementation: 1 TMA double-buffered tiles, 0 synchronous tiles."""
        return self.get_option(_lib.OPT_COL_VARIANT)

    @col_variant.setter
    def col_variant(self, v: int):
        self.set_option(_lib.OPT_COL_VARIANT, v)

    def check(self, stream=None):
        """Synchronise and raise EngineError if a kernel of this plan gave up a bounded wait."""
        _lib.check("es_plan_check", self.lib.es_plan_check(self.handle, _stream_handle(self.device, stream)), self.lib)

    # ------------------------------------------------------------------ per-launch timing
    def profile_enable(self, max_launches: int):
        """Bracket each kernel this plan launches with CUDA events (0 turns it off)."""
        _lib.check("es_profile_enable", self.lib.es_profile_enable(self.handle, int(max_launches)), self.lib)

    def profile_reset(self):
        _lib.check("es_profile_reset", self.lib.es_profile_reset(self.handle), self.lib)

    def profile_read(self) -> dict:
        """{kernel kind: (total ms, launches)} for the launches since the last reset."""
        k = len(_lib.PROF_KINDS)
        ms = (C.c_float * k)()
        cnt = (C.c_int * k)()
        rc = self.lib.es_profile_read(self.handle, ms, cnt, k)
        if rc < 0:
            _lib.check("es_profile_read", rc, self.lib)
        return {name: (float(ms[i]), int(cnt[i])) for i, name in enumerate(_lib.PROF_KINDS) if cnt[i]}

    def close(self):
        if getattr(self, "_h", None) is not None:
            self.lib.es_plan_destroy(self._h)
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
