"""FP64 numpy oracle of the excursion-set hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this module, and only as the checker or the timed CPU baseline.  The product path never
calls it: the CUDA engine fails loudly when its extension is missing.

It restates, per voxel and in float64, what the reference computes on the GPU:

* ``conv_bubbles`` radius loop (Programs/find_HII_bubbles.py:83-92, 121-192)
  - growth rescale ``deltax *= fgrowth`` (l.83-85, float32 as in the reference)
  - forward FFT once (the reference repeats it every radius, l.141-144: same result)
  - ``HII_filter`` (Programs/find_bubbles.cu:12-42); ``ref_compat`` reproduces its
    ``switch`` fall-through (case 0 -> 1 -> 2)
  - normalised inverse FFT and the real part (l.150, 156)
  - ``fcoll_kernel`` erfc (find_bubbles.cu:43-58)
  - mean normalisation when LE is False (l.158-160, 171-173)
  - ``update_kernel`` (find_bubbles.cu:59-71), ``update_sphere_kernel`` (find_bubbles.cu:73-102)
  - ``final_kernel`` (find_bubbles.cu:142-158; launched with the current radius' denom, l.169-175)
* ``delta_T.run`` brightness temperature (Programs/delta_T.py:73-82)
* the power spectrum the reference's ``pbox_kernel`` intends (Programs/delta_T.cu:5-29,
  delta_T.py:87-98): bin = first edge >= |k|, per-bin means of k^3 |g_k|^2 / (2 pi^2 V) and of
  |k|; half-spectrum modes with 0 < i < N/2 count twice (their mirror images).

Parity against the reference itself: the reference (Python 2 + PyCUDA + pyfft + cosmolopy)
cannot run anywhere here, and its repository holds no golden vectors for this path, so the
per-voxel algorithm is PARITY UNPINNED against reference outputs; the host sigma^2 integrator it
depends on is pinned by the reference's ``cosmo_files/sig0.npz`` / ``Del2k.npz`` tables.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erfc

KTOPHAT_FACTOR = 0.413566994     # find_bubbles.cu:34, (9 pi / 2)^(-1/3)
GAUSS_FACTOR = 0.643             # find_bubbles.cu:39


def _fft(backend, workers):
    if backend == "numpy":
        return np.fft.rfftn, np.fft.irfftn
    import scipy.fft as sf
    return (lambda a, **k: sf.rfftn(a, workers=workers, **k),
            lambda a, **k: sf.irfftn(a, workers=workers, **k))


def delta_k(box_len: float) -> float:
    """float32(2 pi / float32(L)) as the reference's DELTA_K (delta_T.py:51-52)."""
    return float(np.float32(2.0 * math.pi / float(np.float32(box_len))))


def k2_grid(n: int) -> np.ndarray:
    """Integer |k / dk|^2 on the half-spectrum grid (n, n, n//2 + 1).

    The wrap follows find_bubbles.cu:21-24: index k > n/2 maps to k - n, so the Nyquist index
    n/2 stays +n/2.
    """
    idx = np.arange(n)
    w = np.where(idx > n // 2, idx - n, idx).astype(np.int64)
    i = np.arange(n // 2 + 1, dtype=np.int64)
    return (w[:, None, None] ** 2 + w[None, :, None] ** 2 + i[None, None, :] ** 2)


def rtophat(x):
    """3 (sin x - x cos x) / x^3 in float64, with its Taylor series below x = 1e-2."""
    x = np.asarray(x, dtype=np.float64)
    out = np.empty_like(x)
    small = x < 1e-2
    xs = x[small]
    out[small] = 1.0 - xs * xs / 10.0 + xs ** 4 / 280.0
    xl = x[~small]
    out[~small] = 3.0 * (np.sin(xl) - xl * np.cos(xl)) / xl ** 3
    return out


def window(k2, dk: float, R: float, filter_type: int, ref_compat: bool):
    """Filter W(kR) applied by HII_filter (find_bubbles.cu:26-41) for modes of integer k^2."""
    kR = dk * np.sqrt(np.asarray(k2, dtype=np.float64)) * float(R)
    if not ref_compat:
        if filter_type == 0:
            return rtophat(kR)
        if filter_type == 1:
            return (kR * KTOPHAT_FACTOR <= 1.0).astype(np.float64)
        if filter_type == 2:
            return np.exp(-(kR * GAUSS_FACTOR) ** 2 / 2.0)
        raise ValueError(filter_type)
    # reference switch without break: case 0 falls into case 1 falls into case 2
    W = np.ones_like(kR)
    if filter_type == 0:
        W = np.where(kR > 1e-4, rtophat(kR), 1.0)
    if filter_type in (0, 1):
        kR = kR * KTOPHAT_FACTOR
        W = np.where(kR > 1.0, 0.0, W)
    if filter_type not in (0, 1, 2):
        raise ValueError(filter_type)
    kR = kR * GAUSS_FACTOR
    return W * np.exp(-kR * kR / 2.0)


def _shift(a, s: int, axis: int, periodic: bool):
    """b[p] = a[p - s] along axis, wrapping (periodic) or filling with False."""
    if s == 0:
        return a
    if periodic:
        return np.roll(a, s, axis=axis)
    out = np.zeros_like(a)
    n = a.shape[axis]
    if abs(s) >= n:
        return out
    src = [slice(None)] * a.ndim
    dst = [slice(None)] * a.ndim
    if s > 0:
        src[axis], dst[axis] = slice(0, n - s), slice(s, n)
    else:
        src[axis], dst[axis] = slice(-s, n), slice(0, n + s)
    out[tuple(dst)] = a[tuple(src)]
    return out


def sphere_r2max(R: float, scale: float, ref_compat: bool) -> int:
    """Largest integer squared cell distance painted around a centre (rsq < R^2, cu:97-98)."""
    if ref_compat:
        # the reference passes R in Mpc and compares float rsq < R*R (float32)
        r2 = np.float32(R) * np.float32(R)
        m = int(math.floor(float(r2)))
        while np.float32(m) >= r2:
            m -= 1
        return m
    rc2 = (float(R) / float(scale)) ** 2
    m = int(math.floor(rc2))
    while m >= rc2:
        m -= 1
    return m


def paint_spheres(centers: np.ndarray, r2max: int, periodic: bool) -> np.ndarray:
    """All cells p with |p - c|^2 <= r2max for some centre c (update_sphere_kernel)."""
    if r2max < 0 or not centers.any():
        return np.zeros_like(centers)
    r = int(math.isqrt(r2max))
    dil = [centers]
    for w in range(1, r + 1):
        dil.append(dil[-1] | _shift(centers, w, 2, periodic) | _shift(centers, -w, 2, periodic))
    out = np.zeros_like(centers)
    for dz in range(-r, r + 1):
        for dy in range(-r, r + 1):
            rem = r2max - dz * dz - dy * dy
            if rem < 0:
                continue
            w = math.isqrt(rem)
            out |= _shift(_shift(dil[w], dz, 0, periodic), dy, 1, periodic)
    return out


def conv_bubbles(deltax, setup, *, tol: float = 1e-5, backend: str = "numpy", workers: int = 1,
                 max_radii: int | None = None):
    """Excursion-set ionisation of one box in float64.

    ``setup`` carries the host scalars (radius schedule, denom, delta_c, fc_mean_ps, zeta) that
    the CUDA path receives too.  Returns a dict with

    * ``ionized``: float64 N^3, 1 = ionised, partial values from the final radius;
    * ``exempt``: cells whose flag lies within ``tol`` of the threshold, where float32 and
      float64 may legitimately disagree (the union of spheres around such centres in sphere
      mode);
    * ``means``: per-radius <fcoll> before normalisation.

    ``max_radii`` stops after that many radii (used to time a bounded CPU sample).  With
    ``workers`` > 1 the FFTs use that many threads (scipy backend) and, in centre mode, the window,
    product and erfc run in slabs on a pool of as many threads (same arithmetic per element).
    """
    rfftn, irfftn = _fft(backend, workers)
    n = setup.n
    d = np.asarray(deltax, dtype=np.float32)
    if d.shape != (n, n, n):
        raise ValueError(f"density box must be {(n, n, n)}, got {d.shape}")
    d = (d * np.float32(setup.growth_scale)).astype(np.float64)    # cu: deltax *= fgrowth
    X = rfftn(d)
    k2 = k2_grid(n)
    dk = delta_k(setup.box_len)
    dc = float(setup.deltac32)
    zeta = float(setup.zeta)
    flags = np.zeros((n, n, n), dtype=bool)
    max_margin = np.full((n, n, n), -np.inf)
    sure = np.zeros((n, n, n), dtype=bool)
    maybe = np.zeros((n, n, n), dtype=bool)
    means = []
    ionized = None
    steps = setup.steps if max_radii is None else setup.steps[:max_radii]
    pool = None
    if workers > 1 and setup.update == 0:
        import concurrent.futures as cf
        pool = cf.ThreadPoolExecutor(workers)
        slabs = [(a, b) for a, b in zip(np.linspace(0, n, workers + 1).astype(int)[:-1],
                                        np.linspace(0, n, workers + 1).astype(int)[1:]) if b > a]
    for st in steps:
        if pool is not None:
            # the same arithmetic in slabs along axis 0 on all workers (numpy and scipy release the GIL)
            def shaped(ab, st=st):
                a, b = ab
                return X[a:b] * (window(k2[a:b], dk, float(st.R), setup.filter_type, setup.ref_compat) / float(n) ** 3)
            XW = np.concatenate(list(pool.map(shaped, slabs)))
            dR = irfftn(XW, s=(n, n, n), axes=(0, 1, 2)) * float(n) ** 3

            def fcoll(ab, st=st):
                a, b = ab
                return erfc((dc - dR[a:b]) / float(st.denom))
            f = np.concatenate(list(pool.map(fcoll, slabs)))
        else:
            W = window(k2, dk, float(st.R), setup.filter_type, setup.ref_compat) / float(n) ** 3
            dR = irfftn(X * W, s=(n, n, n), axes=(0, 1, 2)) * float(n) ** 3
            f = erfc((dc - dR) / float(st.denom))
        if pool is not None and not st.final:
            m = float(sum(pool.map(lambda ab: float(f[ab[0]:ab[1]].sum()), slabs))) / f.size
            means.append(m)
            c = float(setup.fc_mean_ps) / m if setup.normalize_mean else 1.0

            def update(ab):
                a, b = ab
                np.maximum(max_margin[a:b], zeta * (f[a:b] * c) - 1.0, out=max_margin[a:b])
            list(pool.map(update, slabs))
            continue
        m = float(np.mean(f))
        means.append(m)
        if setup.normalize_mean:
            f = f * (float(setup.fc_mean_ps) / m)
        margin = zeta * f - 1.0
        if not st.final:
            if setup.update == 0:
                np.maximum(max_margin, margin, out=max_margin)
            else:
                r2 = sphere_r2max(float(st.R), setup.scale, setup.ref_compat)
                per = not setup.ref_compat
                flags |= paint_spheres(margin >= 0.0, r2, per)
                sure |= paint_spheres(margin > tol, r2, per)
                maybe |= paint_spheres(np.abs(margin) <= tol, r2, per)
        else:
            if setup.update == 0:
                flags = max_margin >= 0.0
            ionized = np.where(flags, 1.0, np.where(margin >= 0.0, 1.0, zeta * f))
    if pool is not None:
        pool.shutdown()
    if setup.update == 0:
        flags = max_margin >= 0.0
        exempt = np.abs(max_margin) <= tol
    else:
        exempt = maybe & ~sure
    if ionized is None:      # bounded sample ended before the final radius
        ionized = flags.astype(np.float64)
    return {"ionized": ionized, "flags": flags, "exempt": exempt, "means": np.array(means),
            "max_margin": max_margin if setup.update == 0 else None}


def delta_T(xH, deltax, const_factor: float):
    """delta_T = const * x_HI * (1 + delta) [mK] and its mean (Programs/delta_T.py:73-76)."""
    dT = float(np.float32(const_factor)) * np.asarray(xH, np.float64) * (1.0 + np.asarray(deltax, np.float64))
    return dT, float(np.mean(dT))


def power_spectrum(dT, ave: float, box_len: float, edges, *, dimensional: bool = False,
                   include_k0: bool = False, backend: str = "numpy", workers: int = 1):
    """Spherically binned Delta^2(k) of the normalised delta_T field (delta_T.py:80-98).

    Returns (K, k_ave, ps_ave, count) with K the float32 edges.
    """
    rfftn, _ = _fft(backend, workers)
    dT = np.asarray(dT, dtype=np.float64)
    n = dT.shape[0]
    L = float(np.float32(box_len))
    volume = L ** 3
    g = (dT / ave - 1.0) * volume / n ** 3
    if dimensional:
        g = g * ave
    G = rfftn(g)
    k2 = k2_grid(n)
    dk = delta_k(box_len)
    kmag = dk * np.sqrt(k2.astype(np.float64))
    wgt = np.full(k2.shape, 2.0)
    wgt[:, :, 0] = 1.0
    wgt[:, :, n // 2] = 1.0
    edges64 = np.asarray(edges, dtype=np.float64)
    b = np.searchsorted(edges64, kmag, side="left")     # first edge >= |k| (delta_T.cu:25-26)
    keep = b < len(edges64)
    if not include_k0:
        keep &= k2 > 0
    nb = len(edges64)
    p = kmag ** 3 * np.abs(G) ** 2 / (2.0 * np.pi ** 2 * volume)
    ps = np.bincount(b[keep], weights=(wgt * p)[keep], minlength=nb)
    ks = np.bincount(b[keep], weights=(wgt * kmag)[keep], minlength=nb)
    ct = np.bincount(b[keep], weights=wgt[keep], minlength=nb)
    with np.errstate(invalid="ignore", divide="ignore"):
        k_ave = np.where(ct > 0, ks / ct, 0.0)
        ps_ave = np.where(ct > 0, ps / ct, 0.0)
    return np.asarray(edges, dtype=np.float32), k_ave, ps_ave, ct
