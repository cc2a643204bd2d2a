"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
produce reference answers.  The product package never imports this module.

* ``Oracle`` wraps oracle/g3l_oracle.c (built into oracle/_build/), the C
  restatement of the reference's integrands and hcubature engine.
* ``RefBuild`` wraps oracle/_ref/libg3lref.so, the reference's own CPU path
  built by oracle/build_ref.sh (only where the reference sources exist), or
  oracle/_ref/libg3lref_scaling.so, its SCALING build, when given scaling arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libg3loracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libg3lref.so")
REF_LIB_SCALING = os.path.join(HERE, "_ref", "libg3lref_scaling.so")

_dp = C.POINTER(C.c_double)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("g3l_oracle.c", "precompute.c")]
    deps = srcs + [os.path.join(HERE, "g3l_oracle.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(s)
                                               for s in deps):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp] + srcs + ["-lm"])
        os.replace(tmp, LIB)
    return LIB


def ref_src() -> str:
    """Directory of the reference's sources: G3L_REF_SRC, else the mount point that
    oracle/build_ref.sh (the recipe that compiles them) documents."""
    if os.environ.get("G3L_REF_SRC"):
        return os.environ["G3L_REF_SRC"]
    r = subprocess.run([os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True,
                       text=True)
    return r.stdout.strip()


def build_ref(scaling: bool = False) -> str | None:
    """Build the reference CPU path (and its SCALING build) when its sources are
    present; the requested library's path, or None where it cannot be had."""
    want = REF_LIB_SCALING if scaling else REF_LIB
    src = ref_src()
    if not os.path.exists(os.path.join(src, "NNMap_Model.cu")):
        return want if os.path.exists(want) else None
    if not (os.path.exists(REF_LIB) and os.path.exists(REF_LIB_SCALING)):
        subprocess.check_call([os.path.join(HERE, "build_ref.sh")])
    return want


class _Hod(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("f", "alpha", "mth", "sigma", "mprime", "beta")]


class _Cosmo(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("Om", "OL", "Ob", "s8", "H0", "ns")]


class _Model(C.Structure):
    _fields_ = [("Nz", C.c_int), ("Nm", C.c_int), ("Nk", C.c_int),
                ("zmin", C.c_double), ("zmax", C.c_double), ("mmin", C.c_double),
                ("mmax", C.c_double), ("kmin", C.c_double), ("kmax", C.c_double),
                ("g", _dp), ("p1", _dp), ("p2", _dp), ("w", _dp), ("dwdz", _dp),
                ("hmf", _dp), ("b_h", _dp), ("conc", _dp), ("P_lin", _dp),
                ("rho_bar", _dp), ("nbar1", _dp), ("nbar2", _dp),
                ("hod1", _Hod), ("hod2", _Hod), ("same_pop", C.c_int),
                ("A", C.c_double), ("eps", C.c_double), ("cosmo", _Cosmo),
                ("clamp_k", C.c_int), ("nthreads", C.c_int),
                ("scaling1", _dp), ("scaling2", _dp)]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build_oracle())
        L.orc_model_init.argtypes = [C.POINTER(_Model)]
        L.orc_term.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, _dp, C.c_int, C.c_int,
                               C.c_size_t, C.c_double, _dp, _dp, C.POINTER(C.c_size_t), _dp]
        L.orc_kernel.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int]
        L.orc_kernel.restype = C.c_double
        L.orc_integrand_points.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, _dp, C.c_int,
                                           C.c_int, C.c_size_t, _dp, _dp]
        L.orc_rule75_region.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, _dp, C.c_int,
                                        C.c_int, _dp, _dp, C.c_double, _dp, _dp,
                                        C.POINTER(C.c_int)]
        L.orc_term_bounds.argtypes = [C.POINTER(_Model), C.c_int, _dp, _dp]
        L.orc_apply_prefactor.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, C.c_double]
        L.orc_apply_prefactor.restype = C.c_double
        L.orc_sici.argtypes = [C.c_double, _dp, _dp]
        L.orc_hcubature_v.argtypes = [C.c_uint, C.c_void_p, C.c_void_p, C.c_uint, _dp, _dp,
                                      C.c_size_t, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                      C.POINTER(C.c_size_t)]
        _lib = L
    return _lib


def precompute(cosmo, nz_z, nz_v, zmin, zmax, mmin, mmax, kmin, kmax, N):
    """The restated doPrecomputations pipeline (precompute.c): dict of g, w, dwdz [N] and
    P_lin, conc, hmf, b_h [N, N], z-major."""
    L = lib()
    L.orc_precompute.argtypes = [_dp, _dp, _dp, C.c_int] + [C.c_double] * 6 + [C.c_int] + [_dp] * 7
    c = np.ascontiguousarray(cosmo, dtype=np.float64)
    zz = np.ascontiguousarray(nz_z, dtype=np.float64)
    zv = np.ascontiguousarray(nz_v, dtype=np.float64)
    N = int(N)
    res = {k: np.zeros(N) for k in ("g", "w", "dwdz")}
    res.update({k: np.zeros((N, N)) for k in ("P_lin", "conc", "hmf", "b_h")})
    L.orc_precompute(_ptr(c), _ptr(zz), _ptr(zv), len(zz), zmin, zmax, mmin, mmax, kmin, kmax, N,
                     *[_ptr(res[k]) for k in ("g", "w", "dwdz", "P_lin", "conc", "hmf", "b_h")])
    return res


INTEGRAND_V = C.CFUNCTYPE(C.c_int, C.c_uint, C.c_size_t, _dp, C.c_void_p, C.c_uint, _dp)


def hod_tuple(h) -> tuple:
    """(f, alpha, Mth, sigma, M', beta) from a dict or sequence."""
    if isinstance(h, dict):
        return tuple(float(h[k]) for k in ("f", "alpha", "mth", "sigma", "mprime", "beta"))
    return tuple(float(x) for x in h)


class Oracle:
    """The restated model on one set of tables and two HOD slots."""

    def __init__(self, tables, hod1, hod2=None, same_pop=False, A=0.0, eps=0.0, clamp_k=True,
                 nthreads=0, scaling=None):
        """scaling: None, or (scaling1, scaling2) [Nm] each, the satellite-variance
        rescaling of the reference's SCALING build."""
        L = lib()
        t = tables
        self._keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in t.arrays().items()}
        self.rho_bar = np.zeros(t.Nz)
        self.nbar1 = np.zeros(t.Nz)
        self.nbar2 = np.zeros(t.Nz)
        m = _Model()
        m.Nz, m.Nm, m.Nk = t.Nz, t.Nm, t.Nk
        m.zmin, m.zmax, m.mmin, m.mmax, m.kmin, m.kmax = (t.zmin, t.zmax, t.mmin, t.mmax, t.kmin,
                                                          t.kmax)
        k = self._keep
        m.g, m.p1, m.p2 = _ptr(k["g"]), _ptr(k["p_lens1"]), _ptr(k["p_lens2"])
        m.w, m.dwdz = _ptr(k["w"]), _ptr(k["dwdz"])
        m.hmf, m.b_h, m.conc, m.P_lin = _ptr(k["hmf"]), _ptr(k["b_h"]), _ptr(k["conc"]), _ptr(
            k["P_lin"])
        m.rho_bar, m.nbar1, m.nbar2 = _ptr(self.rho_bar), _ptr(self.nbar1), _ptr(self.nbar2)
        h1 = hod_tuple(hod1)
        h2 = hod_tuple(hod2 if hod2 is not None else hod1)
        m.hod1 = _Hod(*h1)
        m.hod2 = _Hod(*h2)
        m.same_pop = 1 if (same_pop or hod2 is None) else 0
        m.A, m.eps = A, eps
        c = t.cosmo
        m.cosmo = _Cosmo(c.Om, c.OL, c.Ob, c.s8, c.H0, c.ns)
        m.clamp_k = 1 if clamp_k else 0
        m.nthreads = nthreads
        if scaling is not None:
            self._s = [np.ascontiguousarray(a, dtype=np.float64) for a in scaling]
            if any(a.shape != (t.Nm,) for a in self._s):
                raise ValueError("scaling arrays must have Nm entries")
            m.scaling1, m.scaling2 = _ptr(self._s[0]), _ptr(self._s[1])
        self.m = m
        if L.orc_model_init(C.byref(m)):
            raise RuntimeError("orc_model_init failed")
        self.tables = t

    def term(self, kind: int, term: int, th, type1=1, type2=2, maxEval=1_000_000, rtol=1e-4):
        """(raw val, raw err, numEval, scaled result) of one term."""
        L = lib()
        th = np.ascontiguousarray(th, dtype=np.float64)
        val, err, res = C.c_double(), C.c_double(), C.c_double()
        ne = C.c_size_t()
        st = L.orc_term(C.byref(self.m), kind, term, _ptr(th), type1, type2, maxEval, rtol,
                        C.byref(val), C.byref(err), C.byref(ne), C.byref(res))
        if st:
            raise RuntimeError("orc_term failed")
        return val.value, err.value, ne.value, res.value

    def kernel(self, kind, term, th, pt, type1=1, type2=2):
        th = np.ascontiguousarray(th, dtype=np.float64)
        pt = np.ascontiguousarray(pt, dtype=np.float64)
        return lib().orc_kernel(C.byref(self.m), kind, term, _ptr(th), _ptr(pt), type1, type2)

    def integrand(self, kind, term, th, x, type1=1, type2=2):
        """Integrand over an (n, dim) array of log-coordinates."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(x.shape[0])
        th = np.ascontiguousarray(th, dtype=np.float64)
        lib().orc_integrand_points(C.byref(self.m), kind, term, _ptr(th), type1, type2,
                                   x.shape[0], _ptr(x), _ptr(out))
        return out

    def bounds(self, term):
        lo = np.zeros(7)
        hi = np.zeros(7)
        d = lib().orc_term_bounds(C.byref(self.m), term, _ptr(lo), _ptr(hi))
        return lo[:d].copy(), hi[:d].copy()

    def prefactor(self, kind, term, raw):
        return lib().orc_apply_prefactor(C.byref(self.m), kind, term, raw)

    def region(self, kind, term, th, center, halfwidth, vol, type1=1, type2=2):
        th = np.ascontiguousarray(th, dtype=np.float64)
        c = np.ascontiguousarray(center, dtype=np.float64)
        h = np.ascontiguousarray(halfwidth, dtype=np.float64)
        v, e, s = C.c_double(), C.c_double(), C.c_int()
        lib().orc_rule75_region(C.byref(self.m), kind, term, _ptr(th), type1, type2, _ptr(c),
                                _ptr(h), vol, C.byref(v), C.byref(e), C.byref(s))
        return v.value, e.value, s.value


def oracle_hcubature(f_py, dim, xmin, xmax, maxEval, rtol, reqAbs=0.0, use_ref=False):
    """Integrate a Python vectorised integrand f(x: (n, dim)) -> (n,) with the oracle
    engine (or the reference engine when use_ref)."""

    def cb(ndim, npt, x, fdata, fdim, fval):
        xs = np.ctypeslib.as_array(x, shape=(npt * ndim,)).reshape(npt, ndim)
        out = np.ctypeslib.as_array(fval, shape=(npt,))
        out[:] = f_py(xs)
        return 0

    cfun = INTEGRAND_V(cb)
    lo = np.ascontiguousarray(xmin, dtype=np.float64)
    hi = np.ascontiguousarray(xmax, dtype=np.float64)
    val, err = C.c_double(), C.c_double()
    ne = C.c_size_t()
    if use_ref:
        R = ref_lib()
        st = R.ref_hcubature_v(1, C.cast(cfun, C.c_void_p), None, dim, _ptr(lo), _ptr(hi),
                               maxEval, reqAbs, rtol, 0, C.byref(val), C.byref(err), C.byref(ne))
    else:
        st = lib().orc_hcubature_v(1, C.cast(cfun, C.c_void_p), None, dim, _ptr(lo), _ptr(hi),
                                   maxEval, reqAbs, rtol, 0, C.byref(val), C.byref(err),
                                   C.byref(ne))
    if st:
        raise RuntimeError("hcubature failed")
    return val.value, err.value, ne.value


# ---------------------------------------------------------------------------
# the reference's own CPU build
# ---------------------------------------------------------------------------
_ref = {}


def ref_lib(scaling: bool = False):
    """The reference's CPU build, or its SCALING build (NNMap only)."""
    if scaling not in _ref:
        path = build_ref(scaling)
        if path is None:
            raise FileNotFoundError("reference CPU build unavailable")
        R = C.CDLL(path)
        if scaling:
            R.ref_nnmap_create_scaled.restype = C.c_void_p
            R.ref_nnmap_create_scaled.argtypes = ([_dp] + [C.c_double] * 6 + [C.c_int] +
                                                  [_dp] * 11 +
                                                  [_dp, _dp, C.c_int, C.c_double, C.c_double])
        else:
            R.ref_nnmap_create.restype = C.c_void_p
            R.ref_nnmap_create.argtypes = ([_dp] + [C.c_double] * 6 + [C.c_int] + [_dp] * 9 +
                                           [_dp, _dp, C.c_int, C.c_double, C.c_double])
        R.ref_nnmap_destroy.argtypes = [C.c_void_p]
        R.ref_nnmap_densities.argtypes = [C.c_void_p, _dp, _dp, _dp]
        R.ref_nnmap_term.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, C.c_int, C.c_size_t,
                                     C.c_double, _dp, _dp, C.POINTER(C.c_size_t)]
        R.ref_nnmap_method.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, C.c_int]
        R.ref_nnmap_method.restype = C.c_double
        R.ref_nnmap_kernel.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int, C.c_int]
        R.ref_nnmap_kernel.restype = C.c_double
        R.ref_hcubature_v.argtypes = [C.c_uint, C.c_void_p, C.c_void_p, C.c_uint, _dp, _dp,
                                      C.c_size_t, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                      C.POINTER(C.c_size_t)]
        R.ref_sici.argtypes = [C.c_double, _dp, _dp]
        R.ref_function_read.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_double,
                                        C.c_double, C.c_int, _dp]
        R.ref_function2d_read.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_double,
                                          C.c_double, C.c_double, C.c_double, _dp]
        R.ref_params_read.argtypes = [C.c_char_p, _dp]
        R.ref_cosmology_read.argtypes = [C.c_char_p, _dp]
        if scaling:
            _ref[scaling] = R
            return R
        R.ref_nmapmap_create.restype = C.c_void_p
        R.ref_nmapmap_create.argtypes = ([_dp] + [C.c_double] * 6 + [C.c_int] + [_dp] * 8 +
                                         [_dp])
        R.ref_nmapmap_destroy.argtypes = [C.c_void_p]
        R.ref_nmapmap_densities.argtypes = [C.c_void_p, _dp, _dp]
        R.ref_nmapmap_term.argtypes = [C.c_void_p, C.c_int, _dp, C.c_size_t, C.c_double, _dp,
                                       _dp, C.POINTER(C.c_size_t)]
        R.ref_nmapmap_method.argtypes = [C.c_void_p, C.c_int, _dp]
        R.ref_nmapmap_method.restype = C.c_double
        R.ref_nmapmap_kernel.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        R.ref_nmapmap_kernel.restype = C.c_double
        _ref[scaling] = R
    return _ref[scaling]


class RefBuild:
    """The reference's NNMap_Model (kind 0) or NMapMap_Model (kind 1) on square tables."""

    def __init__(self, tables, hod1, hod2=None, same_pop=False, A=0.0, eps=0.0, kind=0,
                 scaling=None):
        """scaling: None, or (scaling1, scaling2) [N] each: the SCALING build's
        constructor (NNMap only)."""
        t = tables
        if not (t.Nz == t.Nm == t.Nk):
            raise ValueError("the reference model needs Nz == Nm == Nk")
        if scaling is not None and kind != 0:
            raise ValueError("the SCALING build has the NNMap model only")
        R = ref_lib(scaling is not None)
        self.R = R
        self.kind = kind
        self._keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in t.arrays().items()}
        self._cosmo = t.cosmo.as_array()
        k = self._keep
        h1 = np.array(hod_tuple(hod1))
        h2 = np.array(hod_tuple(hod2 if hod2 is not None else hod1))
        self._h = (h1, h2)
        N = t.Nz
        if scaling is not None:
            self._s = [np.ascontiguousarray(a, dtype=np.float64) for a in scaling]
            if any(a.shape != (N,) for a in self._s):
                raise ValueError("scaling arrays must have N entries")
            self.h = R.ref_nnmap_create_scaled(_ptr(self._cosmo), t.zmin, t.zmax, t.kmin,
                                               t.kmax, t.mmin, t.mmax, N, _ptr(k["g"]),
                                               _ptr(k["p_lens1"]), _ptr(k["p_lens2"]),
                                               _ptr(k["w"]), _ptr(k["dwdz"]), _ptr(k["hmf"]),
                                               _ptr(k["P_lin"]), _ptr(k["b_h"]),
                                               _ptr(k["conc"]), _ptr(self._s[0]),
                                               _ptr(self._s[1]), _ptr(h1), _ptr(h2),
                                               1 if (same_pop or hod2 is None) else 0, A, eps)
        elif kind == 0:
            self.h = R.ref_nnmap_create(_ptr(self._cosmo), t.zmin, t.zmax, t.kmin, t.kmax, t.mmin,
                                        t.mmax, N, _ptr(k["g"]), _ptr(k["p_lens1"]),
                                        _ptr(k["p_lens2"]), _ptr(k["w"]), _ptr(k["dwdz"]),
                                        _ptr(k["hmf"]), _ptr(k["P_lin"]), _ptr(k["b_h"]),
                                        _ptr(k["conc"]), _ptr(h1), _ptr(h2),
                                        1 if (same_pop or hod2 is None) else 0, A, eps)
        else:
            self.h = R.ref_nmapmap_create(_ptr(self._cosmo), t.zmin, t.zmax, t.kmin, t.kmax,
                                          t.mmin, t.mmax, N, _ptr(k["g"]), _ptr(k["p_lens1"]),
                                          _ptr(k["w"]), _ptr(k["dwdz"]), _ptr(k["hmf"]),
                                          _ptr(k["P_lin"]), _ptr(k["b_h"]), _ptr(k["conc"]),
                                          _ptr(h1))
        self.N = N

    def densities(self):
        rho = np.zeros(self.N)
        n1 = np.zeros(self.N)
        n2 = np.zeros(self.N)
        if self.kind == 0:
            self.R.ref_nnmap_densities(self.h, _ptr(rho), _ptr(n1), _ptr(n2))
        else:
            self.R.ref_nmapmap_densities(self.h, _ptr(rho), _ptr(n1))
        return rho, n1, n2

    def term(self, term, th, type1=1, type2=2, maxEval=1_000_000, rtol=1e-4):
        th = np.ascontiguousarray(th, dtype=np.float64)
        val, err = C.c_double(), C.c_double()
        ne = C.c_size_t()
        if self.kind == 0:
            st = self.R.ref_nnmap_term(self.h, term, _ptr(th), type1, type2, maxEval, rtol,
                                       C.byref(val), C.byref(err), C.byref(ne))
        else:
            st = self.R.ref_nmapmap_term(self.h, term, _ptr(th), maxEval, rtol, C.byref(val),
                                         C.byref(err), C.byref(ne))
        if st:
            raise RuntimeError("reference hcubature_v failed")
        return val.value, err.value, ne.value

    def method(self, term, th, type1=1, type2=2):
        th = np.ascontiguousarray(th, dtype=np.float64)
        if self.kind == 0:
            return self.R.ref_nnmap_method(self.h, term, _ptr(th), type1, type2)
        return self.R.ref_nmapmap_method(self.h, term, _ptr(th))

    def kernel(self, term, th, pt, type1=1, type2=2):
        th = np.ascontiguousarray(th, dtype=np.float64)
        pt = np.ascontiguousarray(pt, dtype=np.float64)
        if self.kind == 0:
            return self.R.ref_nnmap_kernel(self.h, term, _ptr(th), _ptr(pt), type1, type2)
        return self.R.ref_nmapmap_kernel(self.h, term, _ptr(th), _ptr(pt))

    def close(self):
        if self.h:
            if self.kind == 0:
                self.R.ref_nnmap_destroy(self.h)
            else:
                self.R.ref_nmapmap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
