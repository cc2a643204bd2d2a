"""Python front-end of libg3lgpu.so (ctypes over the C ABI in include/g3l_gpu.h).

This module mirrors the reference's model interface for the hot path:

* ``NNMapModel``   ~ g3lhalo::NNMap_Model   (src/NNMap_Model.h:124-241)
* ``NMapMapModel`` ~ g3lhalo::NMapMap_Model (src/NMapMap_Model.h:115-168)

with the per-term methods ``NNMap_1h/2h/3h``, ``NNMap`` and ``calculateAll``,
plus batched forms that integrate many (triplet, term) pairs in one launch.
Every computation runs in the CUDA library; there is no CPU fallback: if the
library cannot be loaded or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

FP64 = 0
MIXED = 1
NNMAP = 0
NMAPMAP = 1

STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "POOL", 5: "NONFINITE",
          6: "CANCELLED", 7: "ROUNDS", 8: "NO_DEVICE", 9: "BUSY", 10: "DEADLINE"}
# statuses of a finished call whose per-integral results are still returned
_PARTIAL = (4, 5, 6, 7, 10)

_dp = C.POINTER(C.c_double)


class Tables(C.Structure):
    _fields_ = [("Nz", C.c_int), ("Nm", C.c_int), ("Nk", C.c_int),
                ("zmin", C.c_double), ("zmax", C.c_double), ("mmin", C.c_double),
                ("mmax", C.c_double), ("kmin", C.c_double), ("kmax", C.c_double),
                ("g", _dp), ("p_lens1", _dp), ("p_lens2", _dp), ("w", _dp), ("dwdz", _dp),
                ("hmf", _dp), ("b_h", _dp), ("conc", _dp), ("P_lin", _dp),
                ("Om", C.c_double), ("OL", C.c_double), ("Ob", C.c_double),
                ("sigma8", C.c_double), ("H0", C.c_double), ("ns", C.c_double),
                ("clamp_k", C.c_int)]


class Integral(C.Structure):
    _fields_ = [("kind", C.c_int), ("term", C.c_int), ("hod1", C.c_int), ("hod2", C.c_int),
                ("theta", C.c_double * 3), ("rtol", C.c_double), ("max_eval", C.c_uint64)]


class Result(C.Structure):
    _fields_ = [("val", C.c_double), ("err", C.c_double), ("result", C.c_double),
                ("neval", C.c_uint64), ("status", C.c_int32), ("rounds", C.c_int32)]


# numpy views of the item and result structs (same fields, offsets and size), so that a
# batch is converted with array operations instead of a Python loop per integral
INTEGRAL_DT = np.dtype([("kind", "i4"), ("term", "i4"), ("hod1", "i4"), ("hod2", "i4"),
                        ("theta", "f8", (3,)), ("rtol", "f8"), ("max_eval", "u8")])
RESULT_DT = np.dtype([("val", "f8"), ("err", "f8"), ("result", "f8"), ("neval", "u8"),
                      ("status", "i4"), ("rounds", "i4")])
for _ct, _dt in ((Integral, INTEGRAL_DT), (Result, RESULT_DT)):
    assert C.sizeof(_ct) == _dt.itemsize
    assert all(getattr(_ct, f).offset == _dt.fields[f][1] for f in _dt.names)


class ServerStats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("queued", C.c_int32), ("running_integrals", C.c_int32),
                ("free_regions", C.c_uint64)]


class PrecomputeIn(C.Structure):
    _fields_ = [("cosmo", C.c_double * 6), ("nz_z", _dp), ("nz_v", _dp), ("n_nz", C.c_int),
                ("zmin", C.c_double), ("zmax", C.c_double), ("mmin", C.c_double),
                ("mmax", C.c_double), ("kmin", C.c_double), ("kmax", C.c_double),
                ("nbins", C.c_int)]


class PrecomputeOut(C.Structure):
    _fields_ = [("g", _dp), ("w", _dp), ("dwdz", _dp), ("P_lin", _dp), ("conc", _dp),
                ("hmf", _dp), ("b_h", _dp), ("amplitude", C.c_double), ("device_ms", C.c_double),
                ("integrals", C.c_longlong), ("points", C.c_longlong)]


class Options(C.Structure):
    _fields_ = [("eval_blocks_per_sm", C.c_int), ("eval_warps_per_block", C.c_int),
                ("use_graph", C.c_int), ("max_rounds", C.c_int), ("unlimited_pool", C.c_uint64),
                ("small_arg", C.c_double), ("unc_eps_rel", C.c_double),
                ("unc_tau_abs", C.c_double), ("unc_tau_impact", C.c_double),
                ("unc_tau_sel", C.c_double), ("unc_tau_val", C.c_double),
                ("unc_eps_val", C.c_double), ("unc_eps_sel", C.c_double),
                ("evalmx_variant", C.c_int * 6), ("deadline_ms", C.c_double),
                ("unc_thr", C.c_double), ("unc_tau_thr", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("rounds", C.c_uint64),
                ("regions_evaluated", C.c_uint64), ("points_evaluated", C.c_uint64),
                ("tie_fallbacks", C.c_uint64), ("small_arg_fp64", C.c_uint64),
                ("device_ms", C.c_double), ("eval_ms", C.c_double),
                ("escalated", C.c_uint64), ("deferred", C.c_uint64), ("polished", C.c_uint64),
                ("group_ms", C.c_double * 6), ("group_points", C.c_uint64 * 6),
                ("reeval_ms", C.c_double), ("select_ms", C.c_double),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("escalated_full", C.c_uint64), ("thr_checks", C.c_uint64)]


INTEGRAND_V = C.CFUNCTYPE(C.c_int, C.c_uint, C.c_size_t, _dp, C.c_void_p, C.c_uint, _dp)

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libg3lgpu.so, building it first if it is missing or stale."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(path)
            L.g3l_ctx_create.argtypes = [C.POINTER(Tables), C.c_int, C.POINTER(C.c_void_p)]
            L.g3l_ctx_destroy.argtypes = [C.c_void_p]
            L.g3l_set_hod.argtypes = [C.c_void_p, C.c_int, _dp]
            L.g3l_set_hods.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp]
            L.g3l_set_correlation.argtypes = [C.c_void_p, C.c_double, C.c_double]
            L.g3l_set_scaling.argtypes = [C.c_void_p, C.c_int, _dp]
            L.g3l_get_densities.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
            L.g3l_eval.argtypes = [C.c_void_p, C.POINTER(Integral), C.c_int, C.c_int,
                                   C.POINTER(Result)]
            L.g3l_submit.argtypes = [C.c_void_p, C.POINTER(Integral), C.c_int, C.c_int,
                                     C.POINTER(C.c_int64)]
            L.g3l_poll.argtypes = [C.c_void_p, C.c_int64, C.POINTER(Result), C.c_int]
            L.g3l_cancel.argtypes = [C.c_void_p, C.c_int64]
            L.g3l_server_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_int,
                                            C.POINTER(C.c_void_p)]
            L.g3l_server_destroy.argtypes = [C.c_void_p]
            L.g3l_server_destroy.restype = None
            L.g3l_server_submit.argtypes = [C.c_void_p, C.POINTER(Integral), C.c_int,
                                            C.POINTER(C.c_int64)]
            L.g3l_server_poll.argtypes = [C.c_void_p, C.c_int64, C.POINTER(Result), C.c_int, _dp]
            L.g3l_server_cancel.argtypes = [C.c_void_p, C.c_int64]
            L.g3l_server_info.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
            L.g3l_get_options.argtypes = [C.c_void_p, C.POINTER(Options)]
            L.g3l_set_options.argtypes = [C.c_void_p, C.POINTER(Options)]
            L.g3l_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
            L.g3l_last_error.restype = C.c_char_p
            L.g3l_measure_peaks.argtypes = [C.c_void_p, _dp, _dp]
            L.g3l_debug_region.argtypes = [C.c_void_p, C.POINTER(Integral), _dp,
                                           C.POINTER(C.c_int), C.c_int, _dp, _dp]
            L.g3l_eval_cancel.argtypes = [C.c_void_p]
            L.g3l_eval_static.argtypes = [C.c_void_p, C.POINTER(Integral), C.c_int, C.c_int,
                                          C.POINTER(Result)]
            L.g3l_autotune.argtypes = [C.c_void_p, C.POINTER(Integral), C.c_int,
                                       C.POINTER(C.c_int), _dp]
            L.g3l_debug_pool.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp,
                                         C.POINTER(C.c_int), _dp, _dp, C.POINTER(C.c_int),
                                         C.POINTER(C.c_float), C.POINTER(C.c_int)]
            L.g3l_host_densities.argtypes = [C.POINTER(Tables), _dp, _dp, _dp]
            L.g3l_hcubature_v.argtypes = [C.c_uint, C.c_void_p, C.c_void_p, C.c_uint, _dp, _dp,
                                          C.c_size_t, C.c_double, C.c_double, C.c_int, _dp, _dp]
            L.g3l_eval_terms.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_double, C.c_uint64, C.c_int, _dp, _dp, _dp,
                                         C.POINTER(C.c_uint64)]
            L.g3l_precompute_tables.argtypes = [C.POINTER(PrecomputeIn), C.c_int,
                                                C.POINTER(PrecomputeOut)]
            L.g3l_read_function.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_double,
                                            C.c_double, C.c_int, _dp]
            L.g3l_read_function2d.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_double,
                                              C.c_double, C.c_double, C.c_double, _dp]
            L.g3l_read_hod_params.argtypes = [C.c_char_p, _dp]
            L.g3l_read_cosmology.argtypes = [C.c_char_p, _dp]
            L.g3l_read_triplets.argtypes = [C.c_char_p, _dp, C.c_int, C.POINTER(C.c_int)]
            _lib = L
    return _lib


class G3LError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%s): %s" % (STATUS.get(status, status), status, msg))
        self.status = status


def _check(st):
    if st != 0:
        raise G3LError(st, lib().g3l_last_error().decode(errors="replace"))


def _ptr(a):
    return a.ctypes.data_as(_dp)


def make_ctables(t, clamp_k=True):
    """C table struct from a tables.Tables; returns (struct, keep-alive arrays)."""
    keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in t.arrays().items()}
    c = t.cosmo
    ct = Tables(Nz=t.Nz, Nm=t.Nm, Nk=t.Nk, zmin=t.zmin, zmax=t.zmax, mmin=t.mmin, mmax=t.mmax,
                kmin=t.kmin, kmax=t.kmax, g=_ptr(keep["g"]), p_lens1=_ptr(keep["p_lens1"]),
                p_lens2=_ptr(keep["p_lens2"]), w=_ptr(keep["w"]), dwdz=_ptr(keep["dwdz"]),
                hmf=_ptr(keep["hmf"]), b_h=_ptr(keep["b_h"]), conc=_ptr(keep["conc"]),
                P_lin=_ptr(keep["P_lin"]), Om=c.Om, OL=c.OL, Ob=c.Ob, sigma8=c.s8, H0=c.H0,
                ns=c.ns, clamp_k=1 if clamp_k else 0)
    return ct, keep


def host_densities(tables, hod):
    """rho_bar(z), n_bar(z) of one HOD with the library's host integrator (no GPU needed)."""
    ct, keep = make_ctables(tables)
    rho = np.zeros(tables.Nz)
    nb = np.zeros(tables.Nz)
    h = np.ascontiguousarray(hod, dtype=np.float64)
    _check(lib().g3l_host_densities(C.byref(ct), _ptr(h), _ptr(rho), _ptr(nb)))
    return rho, nb


def precompute_tables(cosmo, nz_z, nz_v, zmin, zmax, mmin, mmax, kmin, kmax, nbins, device=0):
    """The reference's doPrecomputations on the device (g3l_precompute_tables).

    cosmo: [Om, OL, Ob, sigma8, H0, ns]; nz_z / nz_v: the source redshift distribution.
    Returns a dict of g, w, dwdz [nbins] and P_lin, conc, hmf, b_h [nbins, nbins]
    (z-major), plus amplitude, device_ms, integrals and points."""
    N = int(nbins)
    zz = np.ascontiguousarray(nz_z, dtype=np.float64)
    zv = np.ascontiguousarray(nz_v, dtype=np.float64)
    if zz.shape != zv.shape or zz.ndim != 1:
        raise ValueError("nz_z and nz_v must be 1-D arrays of one length")
    res = {k: np.empty(N) for k in ("g", "w", "dwdz")}
    res.update({k: np.empty((N, N)) for k in ("P_lin", "conc", "hmf", "b_h")})
    pin = PrecomputeIn(cosmo=(C.c_double * 6)(*[float(x) for x in cosmo]), nz_z=_ptr(zz),
                       nz_v=_ptr(zv), n_nz=len(zz), zmin=zmin, zmax=zmax, mmin=mmin, mmax=mmax,
                       kmin=kmin, kmax=kmax, nbins=N)
    pout = PrecomputeOut(**{k: _ptr(v) for k, v in res.items()})
    _check(lib().g3l_precompute_tables(C.byref(pin), device, C.byref(pout)))
    res.update(amplitude=pout.amplitude, device_ms=pout.device_ms, integrals=pout.integrals,
               points=pout.points)
    return res


def precomputed_tables(cosmo, nz_z, nz_v, zmin, zmax, mmin, mmax, kmin, kmax, nbins, p_lens1,
                       p_lens2=None, device=0):
    """A tables.Tables for the model from precompute_tables and the lens redshift
    distributions p_lens1/2 [nbins] on the same z grid (the inputs the reference's drivers
    read next to the precomputed files)."""
    from .tables import Cosmology, Tables
    r = precompute_tables(cosmo, nz_z, nz_v, zmin, zmax, mmin, mmax, kmin, kmax, nbins, device)
    c = [float(x) for x in cosmo]
    p1 = np.ascontiguousarray(p_lens1, dtype=np.float64)
    p2 = p1 if p_lens2 is None else np.ascontiguousarray(p_lens2, dtype=np.float64)
    return Tables(Nz=nbins, Nm=nbins, Nk=nbins, zmin=zmin, zmax=zmax, mmin=mmin, mmax=mmax,
                  kmin=kmin, kmax=kmax,
                  cosmo=Cosmology(Om=c[0], OL=c[1], Ob=c[2], s8=c[3], h=c[4] / 100.0, ns=c[5],
                                  H0_value=c[4]),
                  g=r["g"], p_lens1=p1, p_lens2=p2, w=r["w"], dwdz=r["dwdz"], hmf=r["hmf"],
                  P_lin=r["P_lin"], b_h=r["b_h"], conc=r["conc"],
                  meta={"precompute": {k: r[k] for k in ("amplitude", "device_ms", "integrals",
                                                         "points")}})


def hcubature_v(f, dim, xmin, xmax, max_eval=0, rtol=1e-4, reqabs=0.0):
    """The library's host hcubature_v with a Python vectorised integrand f(x[n, dim])."""
    def cb(ndim, npt, x, fdata, fdim, fval):
        xs = np.ctypeslib.as_array(x, shape=(npt * ndim,)).reshape(npt, ndim)
        np.ctypeslib.as_array(fval, shape=(npt,))[:] = f(xs)
        return 0
    cf = INTEGRAND_V(cb)
    lo = np.ascontiguousarray(xmin, dtype=np.float64)
    hi = np.ascontiguousarray(xmax, dtype=np.float64)
    val, err = C.c_double(), C.c_double()
    st = lib().g3l_hcubature_v(1, C.cast(cf, C.c_void_p), None, dim, _ptr(lo), _ptr(hi),
                               max_eval, reqabs, rtol, 0, C.byref(val), C.byref(err))
    _check(st)
    return val.value, err.value


class Context:
    """Device-resident tables plus HOD slots; one CUDA stream."""

    def __init__(self, tables, device=0, clamp_k=True):
        L = lib()
        self._ct, self._keep = make_ctables(tables, clamp_k)
        h = C.c_void_p()
        _check(L.g3l_ctx_create(C.byref(self._ct), device, C.byref(h)))
        self.h = h
        self.tables = tables

    def close(self):
        if getattr(self, "h", None):
            lib().g3l_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_hod(self, slot, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        _check(lib().g3l_set_hod(self.h, slot, _ptr(p)))

    def set_hods(self, slots, params):
        """set_hod for many slots at once: their n_bar integrals run in one device launch."""
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(len(sl), 6)
        _check(lib().g3l_set_hods(self.h, len(sl), sl.ctypes.data_as(C.POINTER(C.c_int)),
                                  _ptr(p)))

    def set_correlation(self, A, eps):
        _check(lib().g3l_set_correlation(self.h, A, eps))

    def set_scaling(self, slot, scaling=None):
        """Satellite-variance rescaling s[j] (j < Nm) of a HOD slot; None resets s = 1."""
        if scaling is None:
            _check(lib().g3l_set_scaling(self.h, slot, None))
            return
        a = np.ascontiguousarray(scaling, dtype=np.float64)
        if a.shape != (self.tables.Nm,):
            raise ValueError("scaling needs Nm values")
        _check(lib().g3l_set_scaling(self.h, slot, _ptr(a)))

    def densities(self, slot):
        rho = np.zeros(self.tables.Nz)
        nb = np.zeros(self.tables.Nz)
        _check(lib().g3l_get_densities(self.h, slot, _ptr(rho), _ptr(nb)))
        return rho, nb

    def options(self):
        o = Options()
        _check(lib().g3l_get_options(self.h, C.byref(o)))
        return o

    def set_options(self, **kw):
        o = self.options()
        for k, v in kw.items():
            setattr(o, k, v)
        _check(lib().g3l_set_options(self.h, C.byref(o)))

    def stats(self):
        s = Stats()
        _check(lib().g3l_get_stats(self.h, C.byref(s)))
        out = {}
        for f, _ in Stats._fields_:
            v = getattr(s, f)
            out[f] = list(v) if f in ("group_ms", "group_points") else v
        return out

    def measure_peaks(self):
        """(fp32, fp64) FMA throughput of this device in TFLOP/s."""
        a, b = C.c_double(), C.c_double()
        _check(lib().g3l_measure_peaks(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def debug_region(self, spec, center, levels, precision=FP64):
        """Integrand values at the rule points of one region, and (val, err, split)."""
        items, n = self.make_items([spec])
        dim = spec[1] + 4
        npts = 1 + 4 * dim + 2 * dim * (dim - 1) + (1 << dim)
        c = np.ascontiguousarray(center, dtype=np.float64)
        lv = (C.c_int * dim)(*[int(x) for x in levels])
        vals = np.zeros(npts)
        out = np.zeros(3)
        _check(lib().g3l_debug_region(self.h, items, _ptr(c), lv, precision, _ptr(vals),
                                      _ptr(out)))
        return vals, out

    def debug_pool(self, index):
        """Live regions of item `index` of the last eval: dict of centers [n, dim],
        levels [n, dim], val, err, split."""
        n = C.c_int()
        _check(lib().g3l_debug_pool(self.h, index, 0, None, None, None, None, None, None,
                                    C.byref(n)))
        nr = n.value
        # dimension from the centre count is unknown here; ask with the largest dim
        cen = np.zeros(7 * max(nr, 1))
        lev = np.zeros(7 * max(nr, 1), dtype=np.int32)
        val = np.zeros(max(nr, 1))
        err = np.zeros(max(nr, 1))
        spl = np.zeros(max(nr, 1), dtype=np.int32)
        unc = np.zeros(2 * max(nr, 1), dtype=np.float32)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        _check(lib().g3l_debug_pool(self.h, index, nr, _ptr(cen), ip(lev), _ptr(val), _ptr(err),
                                    ip(spl), unc.ctypes.data_as(C.POINTER(C.c_float)),
                                    C.byref(n)))
        return {"n": nr, "centers": cen, "levels": lev, "val": val[:nr], "err": err[:nr],
                "split": spl[:nr], "unc": unc[:nr], "uval": unc[nr:2 * nr]}

    def autotune(self, specs):
        """Pick the rule-kernel register budget per kind x term on this batch; returns
        (variant per group, ms[6][3])."""
        items, n = self.make_items(specs)
        v = (C.c_int * 6)()
        ms = np.zeros(18)
        _check(lib().g3l_autotune(self.h, items, n, v, _ptr(ms)))
        return list(v), ms.reshape(6, 3)

    @staticmethod
    def make_items(specs):
        """specs: iterable of (kind, term, hod1, hod2, (th1, th2, th3), rtol, max_eval)."""
        specs = list(specs)
        n = len(specs)
        a = np.zeros(max(1, n), dtype=INTEGRAL_DT)
        if n:
            kind, term, h1, h2, th, rtol, me = zip(*specs)
            a["kind"][:n], a["term"][:n], a["hod1"][:n], a["hod2"][:n] = kind, term, h1, h2
            a["theta"][:n] = np.asarray(th, dtype=np.float64).reshape(n, 3)
            a["rtol"][:n] = rtol
            a["max_eval"][:n] = [int(x) for x in me]
        return (Integral * max(1, n)).from_buffer(a), n  # the ctypes array keeps `a` alive

    def eval_terms(self, kind, triplets, hod1, hod2, term_mask=7, rtol=1e-4,
                   max_eval=1_000_000, precision=MIXED):
        """g3l_eval_terms: (val, err, result) [n, 3] and the total evaluation count."""
        th = np.ascontiguousarray(triplets, dtype=np.float64).reshape(-1, 3)
        n = th.shape[0]
        val, err, res = (np.zeros((max(n, 1), 3)) for _ in range(3))
        ne = C.c_uint64()
        st = lib().g3l_eval_terms(self.h, kind, _ptr(th), n, hod1, hod2, term_mask, rtol,
                                  int(max_eval), precision, _ptr(val), _ptr(err), _ptr(res),
                                  C.byref(ne))
        if st != 0 and st not in _PARTIAL:
            _check(st)
        return val[:n], err[:n], res[:n], ne.value

    def eval(self, specs, precision=FP64, check=True):
        """Integrate every spec in one launch; returns a structured numpy array.  Calls
        that end with per-integral statuses (pool, non-finite, cancelled, round cap,
        deadline) return their results; the statuses are in the array."""
        items, n = self.make_items(specs)
        out = (Result * max(1, n))()
        st = lib().g3l_eval(self.h, items, n, precision, out)
        if check and st != 0 and st not in _PARTIAL:
            _check(st)
        return results_to_numpy(out, n)

    def cancel_eval(self):
        """Stop the eval() running on this context from another thread (g3l_eval_cancel):
        its unfinished integrals end with status 6 at the next refinement round."""
        _check(lib().g3l_eval_cancel(self.h))


def results_to_numpy(out, n):
    return np.frombuffer(out, dtype=RESULT_DT, count=n).copy()


class Server:
    """Continuous-batching server on a context (g3l_server_*): submit requests from any
    thread, poll for results; requests that arrive while others run are admitted as
    slots and pool space free up and integrate concurrently with them."""

    def __init__(self, ctx, precision=MIXED, max_items_per_term=1024, pool_regions=1 << 22,
                 rounds_per_launch=4):
        self.ctx = ctx  # keeps the context alive
        h = C.c_void_p()
        _check(lib().g3l_server_create(ctx.h, precision, max_items_per_term, pool_regions,
                                       rounds_per_launch, C.byref(h)))
        self.h = h
        self._n = {}

    def close(self):
        if getattr(self, "h", None):
            lib().g3l_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, specs):
        """specs as for Context.eval; returns a ticket."""
        items, n = Context.make_items(specs)
        t = C.c_int64()
        _check(lib().g3l_server_submit(self.h, items, n, C.byref(t)))
        self._n[t.value] = n
        return t.value

    def poll(self, ticket, wait_ms=-1, check=True):
        """Results (structured array) and latency in ms, or None while running."""
        n = self._n[ticket]
        out = (Result * n)()
        lat = C.c_double()
        st = lib().g3l_server_poll(self.h, ticket, out, wait_ms, C.byref(lat))
        if st == 9:  # G3L_ERR_BUSY
            return None
        del self._n[ticket]
        if check and st != 0 and st not in (4, 5, 6, 7):
            _check(st)
        return results_to_numpy(out, n), lat.value

    def cancel(self, ticket):
        _check(lib().g3l_server_cancel(self.h, ticket))

    def info(self):
        s = ServerStats()
        _check(lib().g3l_server_info(self.h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}


class NNMapModel:
    """The reference's NNMap_Model interface on the GPU engine.

    hod1 / hod2 are parameter vectors {f, alpha, Mth, sigma, M', beta}; passing
    the same object (or hod2=None) reproduces the reference's single-population
    case where both type slots point to one HOD (src/HOD.cu:82).
    The per-term methods use the reference's hard-coded budgets (maxEval 5e6,
    rtol 1e-3, 1e-3, 1e-4; src/NNMap_Model.cu:318,343,368) unless overridden.
    scaling = (scaling1, scaling2) takes the reference's SCALING constructor
    (src/NNMap_Model.cu:103-200): its same-population pair count reads scaling1 for
    both types (src/NNMap_Model.cu:563,808; src/HOD.cu:86-87 use scale1 only), so
    scaling1 goes to both HOD slots and scaling2 is accepted and unused, as there.
    """

    RTOL = {1: 1e-3, 2: 1e-3, 3: 1e-4}
    MAX_EVAL = 5_000_000

    def __init__(self, tables, hod1, hod2=None, A=0.0, epsilon=0.0, precision=FP64, device=0,
                 clamp_k=True, ctx=None, scaling=None):
        self.ctx = ctx or Context(tables, device, clamp_k)
        self.precision = precision
        self.updateHODs(hod1, hod2)
        self.ctx.set_correlation(A, epsilon)
        s1 = None if scaling is None else scaling[0]
        self.ctx.set_scaling(0, s1)
        self.ctx.set_scaling(1, s1)

    def updateHODs(self, hod1, hod2=None):
        same = hod2 is None or hod2 is hod1
        self.ctx.set_hod(0, hod1)
        if not same:
            self.ctx.set_hod(1, hod2)
        self._slot = {1: 0, 2: 0 if same else 1}

    def _spec(self, term, th, type1, type2, rtol=None, max_eval=None):
        return (NNMAP, term, self._slot[type1], self._slot[type2], tuple(th),
                self.RTOL[term] if rtol is None else rtol,
                self.MAX_EVAL if max_eval is None else max_eval)

    def term(self, term, theta1, theta2, theta3, type1=1, type2=2, rtol=None, max_eval=None):
        r = self.ctx.eval([self._spec(term, (theta1, theta2, theta3), type1, type2, rtol,
                                      max_eval)], self.precision)
        return float(r["result"][0])

    def NNMap_1h(self, t1, t2, t3, type1=1, type2=2):
        return self.term(1, t1, t2, t3, type1, type2)

    def NNMap_2h(self, t1, t2, t3, type1=1, type2=2):
        return self.term(2, t1, t2, t3, type1, type2)

    def NNMap_3h(self, t1, t2, t3, type1=1, type2=2):
        return self.term(3, t1, t2, t3, type1, type2)

    def NNMap(self, t1, t2, t3, type1=1, type2=2):
        r = self.batch([(t1, t2, t3)], (1, 2, 3), type1, type2)
        return float(r["result"].sum())

    def batch(self, thetas, terms=(1, 2, 3), type1=1, type2=2, rtol=None, max_eval=None):
        specs = [self._spec(t, th, type1, type2, rtol, max_eval) for th in thetas for t in terms]
        return self.ctx.eval(specs, self.precision)

    def calculateAll(self, thetas1, thetas2, thetas3, hod1, hod2, A=0.0, epsilon=0.0,
                     rtol=None, max_eval=None):
        """N1N2, N1N1, N2N2 blocks of NNMap for every triplet (src/NNMap_Model.cu:382-415)."""
        self.updateHODs(hod1, hod2)
        self.ctx.set_correlation(A, epsilon)
        th = list(zip(thetas1, thetas2, thetas3))
        specs = []
        for (a, b) in ((1, 2), (1, 1), (2, 2)):
            specs += [self._spec(t, x, a, b, rtol, max_eval) for x in th for t in (1, 2, 3)]
        r = self.ctx.eval(specs, self.precision)
        return r["result"].reshape(3 * len(th), 3).sum(axis=1)


class NMapMapModel:
    """The reference's NMapMap_Model interface (one HOD, lens p(z) = p_lens1)."""

    RTOL = {1: 1e-3, 2: 1e-3, 3: 1e-3}
    MAX_EVAL = 5_000_000

    def __init__(self, tables, hod, precision=FP64, device=0, clamp_k=True, ctx=None):
        self.ctx = ctx or Context(tables, device, clamp_k)
        self.precision = precision
        self.updateHOD(hod)

    def updateHOD(self, hod):
        self.ctx.set_hod(0, hod)

    def _spec(self, term, th, rtol=None, max_eval=None):
        return (NMAPMAP, term, 0, 0, tuple(th), self.RTOL[term] if rtol is None else rtol,
                self.MAX_EVAL if max_eval is None else max_eval)

    def term(self, term, t1, t2, t3, rtol=None, max_eval=None):
        r = self.ctx.eval([self._spec(term, (t1, t2, t3), rtol, max_eval)], self.precision)
        return float(r["result"][0])

    def NMapMap_1h(self, t1, t2, t3):
        return self.term(1, t1, t2, t3)

    def NMapMap_2h(self, t1, t2, t3):
        return self.term(2, t1, t2, t3)

    def NMapMap_3h(self, t1, t2, t3):
        return self.term(3, t1, t2, t3)

    def NMapMap(self, t1, t2, t3):
        return float(self.batch([(t1, t2, t3)])["result"].sum())

    def batch(self, thetas, terms=(1, 2, 3), rtol=None, max_eval=None):
        return self.ctx.eval([self._spec(t, th, rtol, max_eval) for th in thetas for t in terms],
                             self.precision)

    def calculateAll(self, thetas1, thetas2, thetas3, hod, rtol=None, max_eval=None):
        self.updateHOD(hod)
        th = list(zip(thetas1, thetas2, thetas3))
        r = self.batch(th, (1, 2, 3), rtol, max_eval)
        return r["result"].reshape(len(th), 3).sum(axis=1)
