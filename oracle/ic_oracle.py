"""CPU restatement of the initial conditions (initialize) -- TEST INFRASTRUCTURE ONLY.

Only the tests import it.

* ``spectrum`` restates init_kernel (initialize.cu:58-95) for the half spectrum drawn from given
  normals, in float32 in the GPU kernel's order: k = m * DELTA_K per axis, |k| = sqrt(kx^2 + ky^2 +
  kz^2), the first table entry K[i] >= |k|, P linearly interpolated, sqrt(P * VOLUME), times
  1/sqrt(2) off the k_z = 0 and N/2 planes and the Hermitian part of the normals on them.  It
  agrees with the GPU bit for bit.
* ``boxes`` restates the rest of initialize.py:83-109 in float64: inverse FFT / BOX_LEN^3 of the
  spectrum (density), of W(kR) times it (smoothed density) and of W(kR) i k_c / k^2 times it
  (displacements, set_velocity initialize.cu:148-190), nearest-cell subsample (initialize.cu:
  133-146).  The window is es_oracle.window.
"""
from __future__ import annotations

import numpy as np

from oracle import es_oracle

SQRT_HALF = np.float32(0.70710678118654752)


def _kaxes(n: int, dk: np.float32):
    m = np.fft.fftfreq(n, d=1.0 / n).astype(np.int64)
    kxy = (m.astype(np.float32) * dk).astype(np.float32)
    kz = (np.arange(n // 2 + 1).astype(np.float32) * dk).astype(np.float32)
    return m, kxy, kz


def spectrum(n: int, box_len: float, nre, nim, K, P) -> np.ndarray:
    L = np.float32(box_len)
    dk = np.float32(2.0 * np.pi / float(L))
    vol = np.float32(L * L * L)
    _, kxy, kz = _kaxes(n, dk)
    kx, ky, kzz = kxy[:, None, None], kxy[None, :, None], kz[None, None, :]
    ksq = ((kx * kx).astype(np.float32) + (ky * ky).astype(np.float32)).astype(np.float32)
    ksq = (ksq + (kzz * kzz).astype(np.float32)).astype(np.float32)
    kmag = np.sqrt(ksq).astype(np.float32)
    K = np.asarray(K, np.float32)
    P = np.asarray(P, np.float32)
    i = np.maximum(np.searchsorted(K, kmag, side="left"), 1)
    i = np.minimum(i, len(K) - 1)
    num = ((P[i] - P[i - 1]).astype(np.float32) * (kmag - K[i - 1]).astype(np.float32)).astype(np.float32)
    ps = (P[i - 1] + (num / (K[i] - K[i - 1]).astype(np.float32)).astype(np.float32)).astype(np.float32)
    amp = np.sqrt((ps * vol).astype(np.float32)).astype(np.float32)
    amp = np.where(ksq == 0, np.float32(0), amp).astype(np.float32)
    nre = np.asarray(nre, np.float32)
    nim = np.asarray(nim, np.float32)
    a = (amp * SQRT_HALF).astype(np.float32)
    re = (a * nre).astype(np.float32)
    im = (a * nim).astype(np.float32)
    j = (-np.arange(n)) % n                    # index of -k along the full axes
    for p in (0, n // 2):                      # Hermitian part on the k_z = 0 and N/2 planes
        mr = nre[j][:, j, p]
        mi = nim[j][:, j, p]
        hr = ((nre[:, :, p] + mr).astype(np.float32) * np.float32(0.5)).astype(np.float32)
        hi = ((nim[:, :, p] - mi).astype(np.float32) * np.float32(0.5)).astype(np.float32)
        re[:, :, p] = (amp[:, :, p] * hr).astype(np.float32)
        im[:, :, p] = (amp[:, :, p] * hi).astype(np.float32)
    return re + 1j * im


def subsample(large: np.ndarray, sw: int, pixel_factor: float) -> np.ndarray:
    dim = large.shape[0]
    a = np.arange(sw).astype(np.float32)
    idx = np.floor((a * np.float32(pixel_factor)).astype(np.float32) + np.float32(0.5)).astype(np.int64)
    idx = np.clip(idx, 0, dim - 1)
    return large[np.ix_(idx, idx, idx)]


def boxes(H: np.ndarray, box_len: float, hii_dim: int, R: float, filter_type: int = 0, ref_compat: bool = False):
    """Float64 density, smoothed density and displacement boxes from the half spectrum H."""
    n = H.shape[0]
    L = float(np.float32(box_len))
    dk = float(np.float32(2.0 * np.pi / L))
    m, _, _ = _kaxes(n, np.float32(dk))
    mz = np.arange(n // 2 + 1)
    k2 = m[:, None, None] ** 2 + m[None, :, None] ** 2 + mz[None, None, :] ** 2
    W = es_oracle.window(k2, dk, R, filter_type, ref_compat)
    H = H.astype(np.complex128)
    inv = lambda X: np.fft.irfftn(X, s=(n, n, n), axes=(0, 1, 2)) * (n ** 3) / L ** 3
    pf = np.float32(n) / np.float32(hii_dim)
    out = {"deltax": inv(H), "smoothed": subsample(inv(W * H), hii_dim, pf)}
    ks2 = np.where(k2 == 0, 1, k2) * dk * dk
    comps = (m[:, None, None] * dk, m[None, :, None] * dk, mz[None, None, :] * dk)
    nyq = (m[:, None, None] == -n // 2, m[None, :, None] == -n // 2, mz[None, None, :] == n // 2)
    for c, name in enumerate(("vx", "vy", "vz")):
        f = np.where((k2 == 0) | nyq[c], 0.0, comps[c] / ks2)
        out[name] = subsample(inv(1j * f * W * H), hii_dim, pf)
    return out
