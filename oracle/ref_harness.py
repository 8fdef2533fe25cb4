"""The reference's conv_bubbles driven through its own CUDA kernels -- TEST INFRASTRUCTURE ONLY.

The second oracle of the parity tests: ``conv_bubbles_ref`` follows find_HII_bubbles.py:83-192
line by line, with torch tensors where the reference has PyCUDA gpuarrays and ``torch.fft``
(cuFFT, complex64) where it has pyfft, and launches the reference's kernels from
Programs/find_bubbles.cu as compiled by ``oracle/build_ref.py`` (its own source, its own
templating).  The product never imports this module.

What stands in for what:

* ``gpuarray.to_gpu_async(deltax.astype(np.complex64))`` + ``fftplan.execute`` (l.141-144):
  ``torch.fft.fftn`` of the complex64 box, unnormalised like pyfft's forward transform;
* ``fftplan.execute(delta_d, inverse=True)`` (l.150): ``torch.fft.ifftn``, normalised by 1/N^3
  like pyfft's inverse (its default ``normalize=True``);
* ``delta_d.real`` (l.156): the real part copied into a float32 box, as PyCUDA's ``.real`` does;
* ``gpuarray.sum(fcoll_d).get()/float(N^3)`` (l.159): a float32 device sum (torch's reduction
  order, not PyCUDA's), then float64 division as numpy 1.x promotes a float32 scalar divided by a
  Python float; ``fcoll_d *= fc_mean_ps/fcollmean`` (l.160): the float64 ratio rounded to float32
  (PyCUDA's scalar multiply casts the scalar to the array's type), then a float32 multiply.

The radius schedule, denominators, delta_c and fc_mean_ps are the host scalars the engine
receives (``IonizeSetup``): this harness pins the per-voxel arithmetic, the host FP64 side is
pinned separately (sigma^2 against the reference's cosmo_files tables).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref


class RefKernels:
    """The five kernels of find_bubbles.cu for one (delta_c, zeta, BOX_LEN), via C launchers."""

    def __init__(self, delta_c: float, zeta: float, box_len: float):
        self.path = build_ref.build(delta_c, zeta, box_len)
        self.lib = C.CDLL(str(self.path))
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        for name, args in (("ref_hii_filter", [vp, i, i, f, vp]), ("ref_fcoll", [vp, vp, i, f, vp]),
                           ("ref_update", [vp, vp, i, vp]), ("ref_update_sphere", [vp, vp, i, f, vp]),
                           ("ref_final", [vp, vp, i, vp])):
            fn = getattr(self.lib, name)
            fn.argtypes = args
            fn.restype = C.c_int

    def call(self, name: str, *args):
        rc = getattr(self.lib, name)(*args)
        if rc != 0:
            raise RuntimeError(f"{name}: CUDA error {rc}")


def conv_bubbles_ref(deltax, setup, device="cuda"):
    """find_HII_bubbles.py:83-192 on the GPU with the reference's kernels; returns ``ionized``
    (float32 numpy, 1 = ionised, partial values from the final radius) and the per-radius
    float32 sums of fcoll."""
    import torch

    n = setup.n
    fil = int(setup.filter_type)
    update = int(setup.update)
    LE = not setup.normalize_mean
    k = RefKernels(float(setup.delta_c), float(setup.zeta), float(setup.box_len))
    stream = C.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    ptr = lambda t: C.c_void_p(t.data_ptr())          # noqa: E731

    deltax = np.float32(np.asarray(deltax, dtype=np.float32).copy())     # l.83
    if not LE:
        deltax *= np.float32(setup.growth_scale)                          # l.84-85, fgrowth = deltac/1.686
    ionized = torch.zeros((n, n, n), dtype=torch.float32, device=device)  # l.87
    width = np.int32(n)
    total = float(n) ** 3
    sums = []
    for st in setup.steps:                                                # l.121-190
        R = np.float32(st.R)                                              # l.125
        denom = np.float32(st.denom)                                      # l.126-128
        delta = torch.from_numpy(deltax.astype(np.complex64)).to(device)  # l.141
        fcoll = torch.zeros((n, n, n), dtype=torch.float32, device=device)  # l.142
        delta = torch.fft.fftn(delta)                                     # l.144 (unnormalised)
        k.call("ref_hii_filter", ptr(delta), int(width), fil, C.c_float(float(R)), stream)   # l.147
        delta = torch.fft.ifftn(delta)                                    # l.150 (normalised)
        real = delta.real.contiguous()                                    # delta_d.real, l.156
        k.call("ref_fcoll", ptr(fcoll), ptr(real), int(width), C.c_float(float(denom)), stream)  # l.156 / 169
        s32 = np.float32(fcoll.sum().item())
        sums.append(s32)
        if not LE:                                                        # l.158-160 / 171-173
            fcollmean = np.float64(s32) / total
            fcoll *= float(np.float32(np.float64(np.float32(setup.fc_mean_ps)) / fcollmean))
        if not st.final:
            if update == 0:
                k.call("ref_update", ptr(ionized), ptr(fcoll), int(width), stream)             # l.163
            else:
                k.call("ref_update_sphere", ptr(ionized), ptr(fcoll), int(width), C.c_float(float(R)), stream)  # l.165
        else:
            k.call("ref_final", ptr(ionized), ptr(fcoll), int(width), stream)                  # l.175
    torch.cuda.synchronize(device)
    return ionized.cpu().numpy(), np.array(sums)
