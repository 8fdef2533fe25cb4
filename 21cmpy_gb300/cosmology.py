"""Host-side FP64 cosmology for the excursion-set path.

Everything here runs on the host in float64; only the resulting scalars (rounded to float32)
reach the GPU.  It restates, from published formulas, the third-party ``cosmolopy`` calls and
the ``cosmo_files/sigmas.py`` integrator that the reference path uses:

* ``pb.sig_del(ION_Tvir_MIN, Z)`` (Programs/find_HII_bubbles.py:57) -> :func:`sig_del`:
  sigma_min = sigma(R(M_vir(T_vir, z)), z=0) and delta_c = 1.686 / D(z).
* ``pb.collapse_fraction(sigmamin, deltac)`` (Programs/find_HII_bubbles.py:60) ->
  :func:`collapse_fraction` = erfc(delta_c / sqrt(2 sigma_min^2)).
* ``sig0(R)`` (cosmo_files/sigmas.py:224-232, 176-191, 99-102, 76-78, 54-66, 44-52) ->
  :class:`SigmaTable`.  Same method: Delta^2(k) tabulated on k = exp(arange(-21, 21, 0.1))
  with linear interpolation, integration limits where the integrand exceeds 1e-6 of its
  maximum on ln k = arange(-20, 20, 0.1), then a 1000-point trapezoid in ln k.
* ``pb.power_spectrum`` (cosmo_files/sigmas.py:46) -> :func:`power_spectrum_z0`: A k^n T(k)^2
  with sigma_8 normalisation; transfer function BBKS (Bardeen et al. 1986, eq. G3, with the
  Sugiyama 1995 shape parameter) or the Eisenstein & Hu (1998) zero-baryon fit, eqs. 26-31.
* ``pb.fgrowth`` -> :func:`growth_factor`: Carroll, Press & Turner (1992) eq. 29.
* ``dDdtoverD`` (Programs/cosmo_functions.py:7-21, on cosmolopy's ``fgrowth`` and ``age``) ->
  :func:`growth_rate`, with :func:`hubble` for H(z).
* ``pb.virial_mass`` -> :func:`virial_mass`: Barkana & Loeb (2001) eq. 26, with the 21cmFAST
  mean molecular weight convention (0.59 at T >= 1e4 K, 1.22 below).

The reference uses two different integrators for sigma_min (cosmolopy ``sigma_r``) and for
sigma^2(R) (sigmas.py); here one integrator serves both.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

__all__ = [
    "Cosmology", "PLANCK13", "BASELINE_COSMO", "transfer_bbks", "transfer_eh_nowiggle",
    "power_spectrum_z0", "growth_factor", "growth_rate", "hubble", "virial_mass", "mass_to_radius", "SigmaTable",
    "sig_del", "collapse_fraction", "tophat_window", "brightness_temperature_factor",
]

# critical density today in h^2 Msun / Mpc^3 (3 H0^2 / 8 pi G with H0 = 100 h km/s/Mpc)
RHO_CRIT_H2 = 2.77536627e11
# kilometres per megaparsec (IAU 2012 astronomical unit; parsec = 648000 / pi au)
MPC_KM = 3.0856775814913673e19


@dataclass(frozen=True)
class Cosmology:
    """Cosmological parameters with cosmolopy's key names (Parameter_files/INIT_PARAMS.py:33-44)."""
    omega_M_0: float = 0.315
    omega_b_0: float = 0.0487
    omega_lambda_0: float = 0.685
    h: float = 0.673
    n: float = 0.96
    sigma_8: float = 0.829
    omega_k_0: float = 0.0
    transfer: str = "EH"          # "EH" (cosmolopy default family) or "BBKS"

    @classmethod
    def from_dict(cls, d: dict) -> "Cosmology":
        keys = {f for f in cls.__dataclass_fields__}
        kw = {k: v for k, v in d.items() if k in keys}
        if "omega_lambda_0" not in d and "omega_M_0" in d:
            kw["omega_lambda_0"] = 1.0 - float(d["omega_M_0"]) - float(d.get("omega_k_0", 0.0))
        return cls(**kw)

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k in self.__dataclass_fields__}


# INIT_PARAMS.py:33-42 (Planck 2013 parameters used by the reference)
PLANCK13 = Cosmology()
# The benchmark density fields: P(k) = A k^0.965 T_BBKS(k)^2, Om=0.31, Ob=0.049, h=0.68, s8=0.81
BASELINE_COSMO = Cosmology(omega_M_0=0.31, omega_b_0=0.049, omega_lambda_0=0.69, h=0.68,
                           n=0.965, sigma_8=0.81, transfer="BBKS")


def tophat_window(y):
    """Real-space top-hat window in Fourier space, W(y) = 3 (sin y - y cos y) / y^3.

    Written exactly as cosmo_files/sigmas.py:24 does, so the sigma^2 integrator reproduces the
    reference's tables; callers that need small-y accuracy use the series form instead.
    """
    y = np.asarray(y, dtype=np.float64)
    return 3.0 * (np.sin(y) - y * np.cos(y)) / y ** 3.0


def transfer_bbks(k, cosmo: Cosmology):
    """BBKS transfer function (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3); k in 1/Mpc.

    Shape parameter Gamma = Om h exp(-Ob (1 + sqrt(2h)/Om)) (Sugiyama 1995).
    """
    k = np.asarray(k, dtype=np.float64)
    om, ob, h = cosmo.omega_M_0, cosmo.omega_b_0, cosmo.h
    gamma = om * h * math.exp(-ob * (1.0 + math.sqrt(2.0 * h) / om))
    q = k / (gamma * h)
    q = np.where(q == 0, 1e-300, q)
    return (np.log1p(2.34 * q) / (2.34 * q)
            * (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25)


def transfer_eh_nowiggle(k, cosmo: Cosmology, t_cmb: float = 2.725):
    """Eisenstein & Hu (1998) zero-baryon-oscillation fit, eqs. 26 and 28-31; k in 1/Mpc."""
    k = np.asarray(k, dtype=np.float64)
    om, ob, h = cosmo.omega_M_0, cosmo.omega_b_0, cosmo.h
    omh2 = om * h * h
    obh2 = ob * h * h
    fb = ob / om
    theta = t_cmb / 2.7
    s = 44.5 * math.log(9.83 / omh2) / math.sqrt(1.0 + 10.0 * obh2 ** 0.75)
    alpha = 1.0 - 0.328 * math.log(431.0 * omh2) * fb + 0.38 * math.log(22.3 * omh2) * fb * fb
    gamma_eff = om * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * k * s) ** 4))
    q = k * theta * theta / (gamma_eff * h)
    L0 = np.log(2.0 * math.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def _transfer(k, cosmo: Cosmology):
    if cosmo.transfer.upper() == "BBKS":
        return transfer_bbks(k, cosmo)
    if cosmo.transfer.upper() == "EH":
        return transfer_eh_nowiggle(k, cosmo)
    raise ValueError(f"unknown transfer function {cosmo.transfer!r}")


def _unnormalised_del2(k, cosmo: Cosmology):
    k = np.asarray(k, dtype=np.float64)
    return k ** 3 * k ** cosmo.n * _transfer(k, cosmo) ** 2 / (2.0 * math.pi ** 2)


_NORM_CACHE: dict = {}


def _sigma8_norm(cosmo: Cosmology) -> float:
    """Amplitude A such that sigma(8/h Mpc) = sigma_8 with a real-space top-hat (dense trapz)."""
    key = cosmo
    if key not in _NORM_CACHE:
        lnk = np.linspace(-16.0, 8.0, 40001)
        k = np.exp(lnk)
        r8 = 8.0 / cosmo.h
        y = _unnormalised_del2(k, cosmo) * tophat_window(k * r8) ** 2
        s2 = np.trapezoid(y, lnk)
        _NORM_CACHE[key] = cosmo.sigma_8 ** 2 / s2
    return _NORM_CACHE[key]


def power_spectrum_z0(k, cosmo: Cosmology):
    """Linear matter power spectrum at z = 0 in Mpc^3, P(k) = A k^n T(k)^2 (sigma_8-normalised)."""
    k = np.asarray(k, dtype=np.float64)
    return _sigma8_norm(cosmo) * k ** cosmo.n * _transfer(k, cosmo) ** 2


def del2_z0(k, cosmo: Cosmology):
    """Dimensionless power Delta^2(k) = k^3 P(k) / (2 pi^2) at z = 0 (cosmo_files/sigmas.py:44-49)."""
    k = np.asarray(k, dtype=np.float64)
    return k ** 3 * power_spectrum_z0(k, cosmo) / (2.0 * math.pi ** 2)


def _omegas_z(z: float, cosmo: Cosmology):
    a3 = (1.0 + z) ** 3
    e2 = cosmo.omega_M_0 * a3 + cosmo.omega_k_0 * (1.0 + z) ** 2 + cosmo.omega_lambda_0
    return cosmo.omega_M_0 * a3 / e2, cosmo.omega_lambda_0 / e2


def growth_factor(z: float, cosmo: Cosmology) -> float:
    """Linear growth D(z)/D(0) from Carroll, Press & Turner (1992) eq. 29."""
    def g(zz):
        om, ol = _omegas_z(zz, cosmo)
        return 2.5 * om / (om ** (4.0 / 7.0) - ol + (1.0 + om / 2.0) * (1.0 + ol / 70.0))
    return g(z) / (g(0.0) * (1.0 + z))


def hubble(z: float, cosmo: Cosmology) -> float:
    """H(z) in 1/s: 100 h km/s/Mpc times sqrt(Om (1+z)^3 + Ok (1+z)^2 + OL)."""
    a1 = 1.0 + z
    e2 = cosmo.omega_M_0 * a1 ** 3 + cosmo.omega_k_0 * a1 ** 2 + cosmo.omega_lambda_0
    return 100.0 * cosmo.h / MPC_KM * math.sqrt(e2)


def growth_rate(z: float, cosmo: Cosmology, dz: float = 1e-4) -> float:
    """(dD/dt) / D in 1/s (Programs/cosmo_functions.py:7-21, ``dDdtoverD``): dD/dz over dt/dz over D.

    The reference takes forward differences (step 1e-10) of cosmolopy's growth factor and of the
    age of the universe; here dD/dz is a central difference of the Carroll-Press-Turner D(z) and
    dt/dz = -1 / ((1 + z) H(z)) is exact."""
    dlnd_dz = (growth_factor(z + dz, cosmo) - growth_factor(z - dz, cosmo)) / (2.0 * dz) / growth_factor(z, cosmo)
    return -dlnd_dz * (1.0 + z) * hubble(z, cosmo)


def virial_mass(t_vir: float, z: float, cosmo: Cosmology, mu: float | None = None) -> float:
    """Halo mass [Msun] with virial temperature t_vir at z (Barkana & Loeb 2001, eq. 26)."""
    if mu is None:
        mu = 0.59 if t_vir >= 9.99999e3 else 1.22
    om_z, _ = _omegas_z(z, cosmo)
    d = om_z - 1.0
    delta_c = 18.0 * math.pi ** 2 + 82.0 * d - 39.0 * d * d
    x = t_vir / (1.98e4 * (mu / 0.6) * ((1.0 + z) / 10.0))
    return 1.0e8 / cosmo.h * x ** 1.5 * (cosmo.omega_M_0 * delta_c / (om_z * 18.0 * math.pi ** 2)) ** -0.5


def mass_to_radius(mass: float, cosmo: Cosmology) -> float:
    """Comoving Lagrangian radius [Mpc] enclosing mass [Msun] at the mean matter density."""
    rho_m = cosmo.omega_M_0 * RHO_CRIT_H2 * cosmo.h ** 2
    return (3.0 * mass / (4.0 * math.pi * rho_m)) ** (1.0 / 3.0)


class SigmaTable:
    """sigma^2(R) at z = 0 by the method of cosmo_files/sigmas.py:44-66, 76-78, 99-102, 176-191.

    ``del2`` is either a cosmology (Delta^2 is then tabulated on k = exp(arange(-21, 21, 0.1)),
    sigmas.py:50-52) or a ``(k, Delta2)`` pair such as the reference's ``Del2k.npz``.
    """

    NINT = 1000                                   # sigmas.py:21

    def __init__(self, del2):
        if isinstance(del2, Cosmology):
            k = np.exp(np.arange(-21.0, 21.0, 0.1))
            d2 = del2_z0(k, del2)
        else:
            k, d2 = (np.asarray(a, dtype=np.float64) for a in del2)
        self.k = k
        self.del2 = d2
        self._cache: dict = {}

    def _del2(self, k):
        return np.interp(k, self.k, self.del2)

    def _integrand(self, logk, R):
        k = np.exp(logk)
        return self._del2(k) * tophat_window(R * k) ** 2

    def _limits(self, R):
        logk = np.arange(-20.0, 20.0, 0.1)
        integrand = self._integrand(logk, R)
        mask = np.abs(integrand) > np.max(np.abs(integrand)) * 1.0e-6
        return np.min(logk[mask]), np.max(logk[mask])

    def sigma2(self, R: float) -> float:
        """sigma^2 of the linear field smoothed with a real-space top-hat of radius R [Mpc]."""
        R = float(R)
        if R not in self._cache:
            lo, hi = self._limits(R)
            logk = np.linspace(lo, hi, self.NINT)
            self._cache[R] = float(np.trapezoid(self._integrand(logk, R), logk))
        return self._cache[R]

    __call__ = sigma2


_SIGMA_TABLES: dict = {}


def sigma_table(cosmo: Cosmology) -> SigmaTable:
    if cosmo not in _SIGMA_TABLES:
        _SIGMA_TABLES[cosmo] = SigmaTable(cosmo)
    return _SIGMA_TABLES[cosmo]


def sig_del(t_vir_min: float, z: float, cosmo: Cosmology, table: SigmaTable | None = None):
    """(sigma_min, delta_c): sigma at the T_vir,min halo scale (z=0 linear) and 1.686/D(z)."""
    table = table or sigma_table(cosmo)
    r_min = mass_to_radius(virial_mass(t_vir_min, z, cosmo), cosmo)
    sigma_min = math.sqrt(table.sigma2(r_min))
    delta_c = 1.686 / growth_factor(z, cosmo)
    return sigma_min, delta_c


def collapse_fraction(sigma_min: float, delta_c: float, sigma_mass: float = 0.0, delta: float = 0.0):
    """Press-Schechter conditional collapse fraction erfc((dc - d) / sqrt(2 (s_min^2 - s_M^2)))."""
    from scipy.special import erfc
    return float(erfc((delta_c - delta) / math.sqrt(2.0 * (sigma_min ** 2 - sigma_mass ** 2))))


def brightness_temperature_factor(z: float, cosmo: Cosmology) -> float:
    """27 (Ob h^2/0.023) sqrt(0.15/(Om h^2) (1+z)/10) mK (Programs/delta_T.py:73-74)."""
    h2 = cosmo.h * cosmo.h
    return 27.0 * (cosmo.omega_b_0 * h2 / 0.023) * math.sqrt((0.15 / cosmo.omega_M_0 / h2) * (1.0 + z) / 10.0)
