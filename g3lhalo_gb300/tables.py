"""Synthetic halo-model lookup tables on the reference's binning.

The reference reads these tables from ASCII files produced by its own
precomputation (src/doPrecomputations.cpp, src/Powerspectrum.cpp, src/HMF.cpp,
src/Cosmology.cpp) and resamples them onto its grids (src/Function.cpp:89-105,
src/Function2D.cpp:66-95).  Here they are generated directly on those grids:

* z_i = zmin + i (zmax - zmin) / Nz,                i = 0 .. Nz-1
* m_j = exp(log(mmin) + j log(mmax/mmin) / Nm),     j = 0 .. Nm-1
* k_j = exp(log(kmin) + j log(kmax/kmin) / Nk),     j = 0 .. Nk-1

Physics (flat LCDM, units Mpc, Msun, k in 1/Mpc):
  w(z), dw/dz from E(z); lensing efficiency g(z) of the source distribution
  p(z) ~ z^2 exp(-(z/0.5)^1.5); Gaussian lens p(z); Eisenstein & Hu (1998)
  no-wiggle linear power spectrum normalised to sigma_8 with linear growth;
  Sheth & Tormen (1999) mass function and bias; c(m, z) = 9/(1+z) (m/1e13)^-0.13.

All arrays are float64, z-major for the 2-D tables (hmf[z, m], P_lin[z, k]).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

C_KMS = 299792.458
RHO_CRIT_H2 = 2.77536627e11  # Msun / Mpc^3 / h^2


@dataclass
class Cosmology:
    Om: float = 0.3
    OL: float = 0.7
    Ob: float = 0.045
    s8: float = 0.8
    h: float = 0.7
    ns: float = 0.96
    H0_value: float | None = None  # H0 [km/s/Mpc] as given (a cosmology file), else 100 h

    @property
    def H0(self) -> float:
        return 100.0 * self.h if self.H0_value is None else self.H0_value

    def as_array(self) -> np.ndarray:
        """[Om, OL, Ob, sigma8, H0, ns], the reference's Cosmology value order."""
        return np.array([self.Om, self.OL, self.Ob, self.s8, self.H0, self.ns], dtype=np.float64)


@dataclass
class Tables:
    Nz: int
    Nm: int
    Nk: int
    zmin: float
    zmax: float
    mmin: float
    mmax: float
    kmin: float
    kmax: float
    cosmo: Cosmology
    g: np.ndarray
    p_lens1: np.ndarray
    p_lens2: np.ndarray
    w: np.ndarray
    dwdz: np.ndarray
    hmf: np.ndarray
    P_lin: np.ndarray
    b_h: np.ndarray
    conc: np.ndarray
    meta: dict = field(default_factory=dict)

    def arrays(self):
        return dict(g=self.g, p_lens1=self.p_lens1, p_lens2=self.p_lens2, w=self.w,
                    dwdz=self.dwdz, hmf=self.hmf, P_lin=self.P_lin, b_h=self.b_h,
                    conc=self.conc)


def _E(c: Cosmology, z):
    return np.sqrt(c.Om * (1 + z) ** 3 + c.OL)


def _comoving(c: Cosmology, z):
    """w(z) in Mpc by cumulative Simpson-quality trapezoid on a fine grid."""
    zf = np.linspace(0.0, max(float(np.max(z)), 5.0) * 1.0001, 200001)
    integrand = 1.0 / _E(c, zf)
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (integrand[1:] + integrand[:-1]) * np.diff(zf))])
    return C_KMS / c.H0 * np.interp(z, zf, cum)


def _growth(c: Cosmology, z):
    """Linear growth factor D(z)/D(0) for flat LCDM."""
    def unnorm(zz):
        a = np.linspace(1e-5, 1.0 / (1.0 + zz), 20001)
        Ea = np.sqrt(c.Om / a ** 3 + c.OL)
        integ = 1.0 / (a * Ea) ** 3
        return 2.5 * c.Om * np.sqrt(c.Om * (1 + zz) ** 3 + c.OL) * np.trapezoid(integ, a)
    d0 = unnorm(0.0)
    z = np.atleast_1d(z)
    return np.array([unnorm(float(zz)) for zz in z]) / d0


def _eh_nowiggle(c: Cosmology, k):
    """Eisenstein & Hu (1998) no-wiggle transfer function; k in 1/Mpc."""
    h = c.h
    om = c.Om * h * h
    ob = c.Ob * h * h
    fb = c.Ob / c.Om
    theta = 2.7255 / 2.7
    s = 44.5 * np.log(9.83 / om) / np.sqrt(1 + 10 * ob ** 0.75)
    alpha = 1 - 0.328 * np.log(431 * om) * fb + 0.38 * np.log(22.3 * om) * fb * fb
    gamma_eff = c.Om * h * (alpha + (1 - alpha) / (1 + (0.43 * k * s) ** 4))
    q = k / h * theta ** 2 / gamma_eff
    L0 = np.log(2 * np.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def _tophat(x):
    x = np.asarray(x)
    out = np.empty_like(x)
    small = x < 1e-3
    xs = x[~small]
    out[~small] = 3 * (np.sin(xs) - xs * np.cos(xs)) / xs ** 3
    out[small] = 1 - x[small] ** 2 / 10
    return out


class _Linear:
    """Normalised z=0 linear power spectrum and sigma(M)."""

    def __init__(self, c: Cosmology):
        self.c = c
        self.lnk = np.linspace(np.log(1e-6), np.log(1e4), 8192)
        k = np.exp(self.lnk)
        self.P_un = k ** c.ns * _eh_nowiggle(c, k) ** 2
        R8 = 8.0 / c.h
        s8_un = self._sigma2(R8, self.P_un)
        self.A = c.s8 ** 2 / s8_un
        self.P0 = self.A * self.P_un
        self.rho_m0 = c.Om * RHO_CRIT_H2 * c.h ** 2

    def _sigma2(self, R, P):
        k = np.exp(self.lnk)
        integ = k ** 3 * P * _tophat(k * R) ** 2 / (2 * np.pi ** 2)
        return np.trapezoid(integ, self.lnk)

    def P(self, k):
        return np.exp(np.interp(np.log(k), self.lnk, np.log(self.P0)))

    def sigma(self, M):
        R = (3 * M / (4 * np.pi * self.rho_m0)) ** (1.0 / 3.0)
        return np.sqrt(np.array([self._sigma2(r, self.P0) for r in np.atleast_1d(R)]))


def make_tables(Nz=64, Nm=128, Nk=256, zmin=0.001, zmax=2.0, mmin=1e10, mmax=1e17,
                kmin_h=1e-4, kmax_h=1e3, cosmo: Cosmology | None = None,
                lens1=(0.3, 0.05), lens2=(0.3, 0.05)) -> Tables:
    """Build every table on the reference's grids.

    kmin_h / kmax_h are in h/Mpc and converted to 1/Mpc.  lens1 / lens2 are the
    (mean, sigma) of the Gaussian lens redshift distributions.
    """
    c = cosmo or Cosmology()
    kmin = kmin_h * c.h
    kmax = kmax_h * c.h
    z = zmin + np.arange(Nz) * (zmax - zmin) / Nz
    m = np.exp(np.log(mmin) + np.arange(Nm) * np.log(mmax / mmin) / Nm)
    k = np.exp(np.log(kmin) + np.arange(Nk) * np.log(kmax / kmin) / Nk)

    w = _comoving(c, z)
    dwdz = C_KMS / c.H0 / _E(c, z)

    # source redshift distribution and lensing efficiency
    zs = np.linspace(1e-4, 4.0, 8001)
    ps = zs ** 2 * np.exp(-((zs / 0.5) ** 1.5))
    ps /= np.trapezoid(ps, zs)
    ws = _comoving(c, zs)
    g = np.empty(Nz)
    for i, (zi, wi) in enumerate(zip(z, w)):
        sel = zs >= zi
        g[i] = np.trapezoid(ps[sel] * (ws[sel] - wi) / ws[sel], zs[sel]) if sel.sum() > 1 else 0.0

    def gauss(mu, sig):
        return np.exp(-0.5 * ((z - mu) / sig) ** 2) / (sig * np.sqrt(2 * np.pi))

    p1 = gauss(*lens1)
    p2 = gauss(*lens2)

    lin = _Linear(c)
    D = _growth(c, z)
    P_lin = (D[:, None] ** 2) * lin.P(k)[None, :]

    # Sheth-Tormen mass function and bias
    A_st, a_st, p_st, dc = 0.3222, 0.707, 0.3, 1.686
    sig0 = lin.sigma(m)
    lnm = np.log(m)
    dlnsig = np.gradient(np.log(sig0), lnm)
    hmf = np.empty((Nz, Nm))
    b_h = np.empty((Nz, Nm))
    for i in range(Nz):
        nu = dc / (sig0 * D[i])
        anu2 = a_st * nu * nu
        fnu = A_st * np.sqrt(2 * anu2 / np.pi) * (1 + anu2 ** (-p_st)) * np.exp(-anu2 / 2)
        hmf[i] = lin.rho_m0 / m ** 2 * fnu * (-dlnsig)
        b_h[i] = 1 + (anu2 - 1) / dc + 2 * p_st / (dc * (1 + anu2 ** p_st))
    conc = 9.0 / (1 + z)[:, None] * (m[None, :] / 1e13) ** (-0.13)

    t = Tables(Nz=Nz, Nm=Nm, Nk=Nk, zmin=zmin, zmax=zmax, mmin=mmin, mmax=mmax, kmin=kmin,
               kmax=kmax, cosmo=c, g=g, p_lens1=p1, p_lens2=p2, w=w, dwdz=dwdz,
               hmf=np.ascontiguousarray(hmf), P_lin=np.ascontiguousarray(P_lin),
               b_h=np.ascontiguousarray(b_h), conc=np.ascontiguousarray(conc))
    t.meta = dict(lens1=lens1, lens2=lens2, kmin_h=kmin_h, kmax_h=kmax_h)
    return t
