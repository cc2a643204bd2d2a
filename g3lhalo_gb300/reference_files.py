"""The reference's ASCII inputs, read as its drivers read them.

The drivers src/calculateNNMap.cu, src/calculateNNMap_twoPop.cu and
src/calculateNMapMap.cu take a cosmology file, the binning, one file per lookup
table, HOD parameter files and a file of aperture triplets (src/calculateNNMap.cu:
42-129).  These functions load the same files through the library's native readers
(g3l_read_* in include/g3l_gpu.h), which follow g3lhalo::Function / Function2D /
Params / Cosmology, so a Tables built here holds the arrays the reference's model
receives from the same files.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .api import _check, _ptr, lib
from .tables import Cosmology, Tables
from .workloads import ARCMIN_IN_RAD  # noqa: F401  (the drivers' arcmin -> rad factor)


def _path(p) -> bytes:
    return str(p).encode()


def read_function(path, nbins, vmin, vmax, default=0.0, log_bins=False):
    """A 1-D "x y" table sampled on nbins linear (Function::read) or logarithmic
    (Function::readLog) bins of [vmin, vmax)."""
    out = np.empty(nbins)
    _check(lib().g3l_read_function(_path(path), default, nbins, vmin, vmax,
                                   1 if log_bins else 0, _ptr(out)))
    return out


def read_function2d(path, nbins, min1, max1, min2, max2, default=0.0):
    """A 2-D "x1 x2 y" table on nbins x nbins bins (Function2D::read), shape (nbins, nbins)."""
    out = np.empty(nbins * nbins)
    _check(lib().g3l_read_function2d(_path(path), default, nbins, min1, max1, min2, max2,
                                     _ptr(out)))
    return out.reshape(nbins, nbins)


def read_hod_params(path):
    """A HOD parameter file as {f, alpha, Mth, sigma, M', beta} (the C ABI's slot order)."""
    out = np.empty(6)
    _check(lib().g3l_read_hod_params(_path(path), _ptr(out)))
    return out


def read_cosmology(path) -> Cosmology:
    out = np.empty(6)
    _check(lib().g3l_read_cosmology(_path(path), _ptr(out)))
    return Cosmology(Om=out[0], OL=out[1], Ob=out[2], s8=out[3], h=out[4] / 100.0, ns=out[5],
                     H0_value=out[4])


def read_triplets(path):
    """Aperture triplets in arcmin, shape (n, 3)."""
    n = C.c_int()
    _check(lib().g3l_read_triplets(_path(path), None, 0, C.byref(n)))
    out = np.empty(3 * max(n.value, 1))
    _check(lib().g3l_read_triplets(_path(path), _ptr(out), n.value, C.byref(n)))
    return out[: 3 * n.value].reshape(-1, 3)


def tables_from_files(fn_cosmo, zmin, zmax, kmin, kmax, mmin, mmax, nbins, fn_g, fn_plens1,
                      fn_plens2, fn_w, fn_dwdz, fn_hmf, fn_P_lin, fn_b_h, fn_conc) -> Tables:
    """Tables from the reference driver's inputs, in its argument order
    (src/calculateNNMap.cu:42-72): the z tables on linear bins, hmf, b_h and the
    concentration over (z, m) and P_lin over (z, k), default value 0 everywhere.
    NMapMap's driver passes one lens file: give it as fn_plens1 and fn_plens2."""
    z = lambda fn: read_function(fn, nbins, zmin, zmax)  # noqa: E731
    zm = lambda fn: read_function2d(fn, nbins, zmin, zmax, mmin, mmax)  # noqa: E731
    return Tables(Nz=nbins, Nm=nbins, Nk=nbins, zmin=zmin, zmax=zmax, mmin=mmin, mmax=mmax,
                  kmin=kmin, kmax=kmax, cosmo=read_cosmology(fn_cosmo), g=z(fn_g),
                  p_lens1=z(fn_plens1), p_lens2=z(fn_plens2), w=z(fn_w), dwdz=z(fn_dwdz),
                  hmf=zm(fn_hmf), P_lin=read_function2d(fn_P_lin, nbins, zmin, zmax, kmin, kmax),
                  b_h=zm(fn_b_h), conc=zm(fn_conc))


def scaling_from_file(path, nbins, mmin, mmax):
    """A SCALING array as the reference's driver reads it: Function::read on linear
    bins of [mmin, mmax), default value 1 (src/calculateNNMap_twoPop.cu:88-89,121).
    The model indexes it by the logarithmic mass bin (src/NNMap_Model.cu:556,563)."""
    return read_function(path, nbins, mmin, mmax, default=1.0)
