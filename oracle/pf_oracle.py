"""CPU restatement of the density evolution (perturb_field) -- TEST INFRASTRUCTURE ONLY.

Only the tests import it.  It restates, with numpy float32 operations in the reference's order:

* ``evolve_linear`` -- perturb_field.py:39-50: updated = deltax * D(z) (float32 multiply);
* ``move_mass`` -- perturb_field.cu:90-132 with the velocity scaling and normalisation of
  perturb_field.py:91-101: each DIM^3 cell at ((a + 0.5) / DIM) per axis moves by
  v * (D(z) - D(z_init)) / BOX_LEN of the HII cell it lies in (index floor(a / PIXEL_FACTOR)),
  is scaled to the HII grid, wrapped by repeated +- HII_DIM, truncated to a cell index, and adds
  its mass 1 + D(z_init) delta there; the grid is divided by MASS_FACTOR and 1 is subtracted.
* ``velocities`` -- perturb_field.py:110-125 with set_velocity / filter / subsample
  (perturb_field.cu:39-88): per component c, (dD/dt / D) irfftn(W(kR) i k_c / k^2 rfftn(deltax)) in
  float64 (forward unnormalised, inverse normalised, as pyfft), zero at k = 0 and at the
  component's Nyquist index (the real part of the reference's complex inverse drops it), then the
  nearest-cell subsample.

The reference sums the masses with float atomics (order-dependent); this restatement sums each
cell's float32 mass as a 64-bit fixed-point integer with 32 fraction bits (round half to even),
exactly, which is what the GPU kernel does, so the two agree bit for bit.  Parity against the
reference's own outputs is unpinned: the reference holds no fixtures for this step and cannot run
here.
"""
from __future__ import annotations

import numpy as np

FIX = 2.0 ** 32
WRAP_LIMIT = 64


def evolve_linear(deltax: np.ndarray, growth: float) -> np.ndarray:
    """perturb_field.py:43-47: deltax * fgrowth in float32."""
    return (np.asarray(deltax, np.float32) * np.float32(growth)).astype(np.float32)


def axis_tables(dim: int, hii_dim: int, pixel_factor: float):
    """Positions (a + 0.5) / DIM (double, rounded to float32: perturb_field.cu:104-106) and the HII
    cell floor(a / PIXEL_FACTOR) of every index (float32 division: perturb_field.cu:107-109)."""
    a = np.arange(dim)
    pos = ((a + 0.5) / float(dim)).astype(np.float32)
    hidx = np.floor(a.astype(np.float32) / np.float32(pixel_factor)).astype(np.int64)
    if hidx.min() < 0 or hidx.max() >= hii_dim:
        raise ValueError("pixel factor maps an index outside the HII grid")
    return pos, hidx


def _target(p: np.ndarray, vel: np.ndarray, ds: np.float32, sw: int) -> np.ndarray:
    """perturb_field.cu:111-127 for one axis (float32 throughout, no fused multiply-add)."""
    swf = np.float32(sw)
    f = (p + (vel * ds).astype(np.float32)).astype(np.float32)
    f = (f * swf).astype(np.float32)
    for _ in range(WRAP_LIMIT):
        m = f >= swf
        if not m.any():
            break
        f = np.where(m, (f - swf).astype(np.float32), f)
    for _ in range(WRAP_LIMIT):
        m = f < np.float32(0)
        if not m.any():
            break
        f = np.where(m, (f + swf).astype(np.float32), f)
    i = np.where(np.isfinite(f), f, 0).astype(np.int64)      # truncation toward zero
    i = np.where(i >= sw, i - sw, i)
    i = np.where(i < 0, i + sw, i)
    return np.clip(i, 0, sw - 1)


def move_mass(deltax, vx, vy, vz, init_growth: float, disp_scale: float, pixel_factor: float,
              mass_factor: float, return_sums: bool = False, first_plane: int = 0):
    """Zel'dovich move of a DIM^3 box onto the HII_DIM^3 grid of the velocity boxes.

    deltax may be a slab of consecutive axis-0 planes of the DIM^3 box, starting at `first_plane`
    (DIM is its last extent); only those cells are moved."""
    deltax = np.asarray(deltax, np.float32)
    dim, sw = deltax.shape[2], np.asarray(vx).shape[0]
    pos, hidx = axis_tables(dim, sw, pixel_factor)
    ds = np.float32(disp_scale)
    g0 = np.float32(init_growth)
    acc = np.zeros(sw ** 3, np.float64)                       # integer sums < 2^53 stay exact
    for i in range(deltax.shape[0]):                          # one DIM plane at a time
        a0 = first_plane + i
        h0 = hidx[a0]
        h1, h2 = np.meshgrid(hidx, hidx, indexing="ij")
        vxs = np.asarray(vx, np.float32)[h0][h1, h2]
        vys = np.asarray(vy, np.float32)[h0][h1, h2]
        vzs = np.asarray(vz, np.float32)[h0][h1, h2]
        p1, p2 = np.meshgrid(pos, pos, indexing="ij")
        t0 = _target(np.full_like(p1, pos[a0]), vxs, ds, sw)
        t1 = _target(p1, vys, ds, sw)
        t2 = _target(p2, vzs, ds, sw)
        mass = (np.float32(1) + (g0 * deltax[i]).astype(np.float32)).astype(np.float32)
        q = np.rint(mass.astype(np.float64) * FIX)
        flat = (t0 * sw + t1) * sw + t2
        acc += np.bincount(flat.ravel(), weights=q.ravel(), minlength=sw ** 3)
    sums = acc.astype(np.int64)
    m = (sums.astype(np.float64).astype(np.float32) * np.float32(1.0 / FIX)).astype(np.float32)
    out = ((m / np.float32(mass_factor)).astype(np.float32) - np.float32(1)).astype(np.float32)
    out = out.reshape(sw, sw, sw)
    return (out, sums.reshape(sw, sw, sw)) if return_sums else out


def velocities(deltax, hii_dim: int, box_len: float, R: float, growth_rate: float, pixel_factor: float,
               filter_type: int = 0, ref_compat: bool = False) -> dict:
    """Float64 velocity boxes at the evolved redshift from the DIM^3 density (perturb_field.py:110-125)."""
    from oracle import es_oracle, ic_oracle
    d = np.asarray(deltax, np.float64)
    n = d.shape[0]
    L = float(np.float32(box_len))
    dk = float(np.float32(2.0 * np.pi / L))
    m = np.fft.fftfreq(n, d=1.0 / n).astype(np.int64)
    mz = np.arange(n // 2 + 1)
    k2 = m[:, None, None] ** 2 + m[None, :, None] ** 2 + mz[None, None, :] ** 2
    X = np.fft.rfftn(d) * es_oracle.window(k2, dk, R, filter_type, ref_compat)
    ks2 = np.where(k2 == 0, 1, k2) * dk * dk
    comps = (m[:, None, None] * dk, m[None, :, None] * dk, mz[None, None, :] * dk)
    nyq = (m[:, None, None] == -n // 2, m[None, :, None] == -n // 2, mz[None, None, :] == n // 2)
    out = {}
    for c, name in enumerate(("vx", "vy", "vz")):
        f = np.where((k2 == 0) | nyq[c], 0.0, comps[c] / ks2) * float(np.float32(growth_rate))
        out[name] = ic_oracle.subsample(np.fft.irfftn(1j * f * X, s=(n, n, n), axes=(0, 1, 2)), hii_dim, pixel_factor)
    return out
