"""Generate the golden vectors in tests/golden/ from the reference's own CPU build.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py            # ref_n64.npz
    python tests/golden/make_golden.py --scaling  # ref_scaling_n64.npz
    python tests/golden/make_golden.py --precompute  # ref_precompute.npz
It builds oracle/_ref/libg3lref.so and libg3lref_scaling.so (oracle/build_ref.sh)
from the reference's unmodified sources, drives NNMap_Model / NMapMap_Model /
hcubature_v in memory through oracle/ref_harness.cu, and writes the fixture.  The
tables the vectors were computed on are stored in ref_n64.npz, so the fixtures do
not depend on the table generator being bit-identical across platforms; the
SCALING vectors are computed on the tables read back from that file.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from g3lhalo_gb300 import workloads as W  # noqa: E402
from g3lhalo_gb300.tables import make_tables  # noqa: E402
import pyoracle as P  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "ref_n64.npz")
OUT_SCALING = os.path.join(ROOT, "tests", "golden", "ref_scaling_n64.npz")
OUT_PRECOMPUTE = os.path.join(ROOT, "tests", "golden", "ref_precompute.npz")

# doPrecomputations inputs: (cosmology [Om, OL, Ob, sigma8, H0, ns], zmin, zmax, mmin, mmax,
# kmin, kmax, nbins); the source n(z) is a smooth seeded stand-in for the survey's file
PRECOMPUTE_CASES = [
    ((0.3, 0.7, 0.045, 0.8, 70.0, 0.96), 0.1, 2.0, 1e10, 1e17, 0.01, 1000.0, 16),
    ((0.3089, 0.6911, 0.0486, 0.8159, 67.74, 0.9667), 0.001, 1.5, 1e9, 1e16, 1e-3, 1e4, 12),
]


def source_nz(n=60, zmax=3.0, z0=0.5):
    z = np.linspace(0.0, zmax, n)
    v = z * z * np.exp(-(z / z0) ** 1.5)
    return z, v / (v.sum() * (z[1] - z[0]))

# analytic integrands for the engine-only vectors (Genz test families)
def genz_gauss(x):
    a = np.array([3.0, 2.0, 5.0, 1.5, 4.0, 2.5, 3.5])[: x.shape[1]]
    u = np.array([0.3, 0.6, 0.45, 0.7, 0.2, 0.55, 0.4])[: x.shape[1]]
    return np.exp(-np.sum(a * a * (x - u) ** 2, axis=1))


def genz_osc(x):
    a = np.array([2.0, 1.0, 3.0, 1.5, 2.5, 0.5, 1.2])[: x.shape[1]]
    return np.cos(2 * np.pi * 0.3 + x @ a)


def genz_corner(x):
    a = np.array([1.0, 2.0, 0.5, 1.5, 1.0, 0.7, 1.1])[: x.shape[1]]
    return (1.0 + x @ a) ** (-(x.shape[1] + 1))


ENGINE_CASES = [  # (name, dim, maxEval, rtol)
    ("gauss", 1, 0, 1e-10), ("gauss", 2, 20000, 1e-8), ("gauss", 5, 40000, 1e-6),
    ("osc", 3, 30000, 1e-9), ("osc", 7, 60000, 1e-6), ("corner", 4, 40000, 1e-7),
    ("corner", 6, 50000, 1e-7), ("osc", 1, 0, 1e-12),
]
FUNCS = {"gauss": genz_gauss, "osc": genz_osc, "corner": genz_corner}


def main():
    P.build_ref()
    T = make_tables(Nz=64, Nm=64, Nk=64, kmax_h=1e7 / 0.7)
    h1, h2 = W.hod_default(), W.hod_second()
    out = {f"tab_{k}": v for k, v in T.arrays().items()}
    out["tab_meta"] = np.array([T.Nz, T.Nm, T.Nk, T.zmin, T.zmax, T.mmin, T.mmax, T.kmin, T.kmax])
    out["cosmo"] = T.cosmo.as_array()
    out["hod1"], out["hod2"] = h1, h2

    rng = np.random.default_rng(20261203)
    trip = W.triplets_all()
    thetas = np.array([trip[0], trip[57], trip[219], W.triplets_equal((1.0,))[0]])
    out["thetas"] = thetas

    # --- NNMap model, two populations ---
    R = P.RefBuild(T, h1, h2, kind=0)
    O = P.Oracle(T, h1, h2, clamp_k=False)
    rho, n1, n2 = R.densities()
    out["nn_rho_bar"], out["nn_nbar1"], out["nn_nbar2"] = rho, n1, n2
    for term in (1, 2, 3):
        lo, hi = O.bounds(term)
        x = rng.uniform(lo, hi, size=(48, len(lo)))
        pts = x.copy()
        pts[:, :2] = 10 ** pts[:, :2]
        pts[:, 3:-1] = 10 ** pts[:, 3:-1]
        vals = np.array([[R.kernel(term, thetas[1], p, t1, t2) for (t1, t2) in
                          ((1, 2), (1, 1), (2, 2))] for p in pts])
        out[f"nn_pts_t{term}"] = pts
        out[f"nn_kernel_t{term}"] = vals
    rows = []
    for it, th in enumerate(thetas):
        for term in (1, 2, 3):
            for (t1, t2) in ((1, 2), (1, 1)):
                v, e, n = R.term(term, th, t1, t2, maxEval=60000, rtol=1e-4)
                rows.append([it, term, t1, t2, 60000, v, e, n])
    out["nn_terms"] = np.array(rows, dtype=np.float64)
    stock = [[term, R.method(term, thetas[1], 1, 2)] for term in (1, 2, 3)]
    out["nn_stock"] = np.array(stock)
    R.close()

    # --- NNMap model with one HOD object in both slots ---
    R = P.RefBuild(T, h1, None, kind=0)
    rows = []
    for term in (1, 2, 3):
        v, e, n = R.term(term, thetas[2], 1, 2, maxEval=40000, rtol=1e-4)
        rows.append([2, term, 1, 2, 40000, v, e, n])
    out["nn_same_terms"] = np.array(rows, dtype=np.float64)
    R.close()

    # --- NMapMap model ---
    R = P.RefBuild(T, h2, None, kind=1)
    rho, nb, _ = R.densities()
    out["nm_rho_bar"], out["nm_nbar"] = rho, nb
    for term in (1, 2, 3):
        lo, hi = O.bounds(term)
        x = rng.uniform(lo, hi, size=(48, len(lo)))
        pts = x.copy()
        pts[:, :2] = 10 ** pts[:, :2]
        pts[:, 3:-1] = 10 ** pts[:, 3:-1]
        out[f"nm_pts_t{term}"] = pts
        out[f"nm_kernel_t{term}"] = np.array([R.kernel(term, thetas[0], p) for p in pts])
    rows = []
    for it, th in enumerate(thetas[:3]):
        for term in (1, 2, 3):
            v, e, n = R.term(term, th, maxEval=60000, rtol=1e-4)
            rows.append([it, term, 0, 0, 60000, v, e, n])
    out["nm_terms"] = np.array(rows, dtype=np.float64)
    out["nm_stock"] = np.array([[1, R.method(1, thetas[0])]])
    R.close()

    # --- engine-only vectors on analytic integrands ---
    rows = []
    for ci, (name, dim, me, rtol) in enumerate(ENGINE_CASES):
        v, e, n = P.oracle_hcubature(FUNCS[name], dim, np.zeros(dim), np.ones(dim), me, rtol,
                                     use_ref=True)
        rows.append([ci, dim, me, rtol, v, e, n])
    out["engine"] = np.array(rows)

    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


def scaling_arrays(N):
    """Satellite-variance rescalings per mass bin: scaling1 in [0.6, 1.4] (below 1 the
    same-population pair count goes negative at small N_sat, which the reference does
    not clip), scaling2 a different ramp (the reference never reads it)."""
    j = np.arange(N)
    return 1.0 + 0.4 * np.sin(0.23 * j), 0.7 + 0.02 * j


def main_scaling():
    """Vectors of the reference's SCALING build (NNMap 1- and 2-halo terms)."""
    P.build_ref(scaling=True)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import tables_from_golden  # noqa: E402
    g = dict(np.load(OUT))
    T = tables_from_golden(g)
    h1, h2 = g["hod1"], g["hod2"]
    thetas = g["thetas"]
    s1, s2 = scaling_arrays(T.Nm)
    out = {"scaling1": s1, "scaling2": s2}
    rng = np.random.default_rng(20261204)
    R = P.RefBuild(T, h1, h2, kind=0, scaling=(s1, s2))
    O = P.Oracle(T, h1, h2, clamp_k=False)
    for term in (1, 2):
        lo, hi = O.bounds(term)
        pts = rng.uniform(lo, hi, size=(48, len(lo)))
        pts[:, :2] = 10 ** pts[:, :2]
        pts[:, 3:-1] = 10 ** pts[:, 3:-1]
        out[f"sc_pts_t{term}"] = pts
        out[f"sc_kernel_t{term}"] = np.array(
            [[R.kernel(term, thetas[1], p, t1, t2) for (t1, t2) in ((1, 2), (1, 1), (2, 2))]
             for p in pts])
    rows = []
    for it in (1, 2):
        for term in (1, 2):
            for (t1, t2) in ((1, 1), (2, 2), (1, 2)):
                v, e, n = R.term(term, thetas[it], t1, t2, maxEval=60000, rtol=1e-4)
                rows.append([it, term, t1, t2, 60000, v, e, n])
    out["sc_terms"] = np.array(rows, dtype=np.float64)
    out["sc_stock"] = np.array([[term, R.method(term, thetas[1], 1, 1)] for term in (1, 2)])
    R.close()
    R = P.RefBuild(T, h1, None, kind=0, scaling=(s1, s2))
    rows = []
    for term in (1, 2):
        v, e, n = R.term(term, thetas[0], 1, 2, maxEval=40000, rtol=1e-4)
        rows.append([0, term, 1, 2, 40000, v, e, n])
    out["sc_same_terms"] = np.array(rows, dtype=np.float64)
    R.close()
    np.savez_compressed(OUT_SCALING, **out)
    print("wrote", OUT_SCALING, os.path.getsize(OUT_SCALING), "bytes")


def main_precompute():
    """Tables of the reference's doPrecomputations pipeline (in memory, no 6-digit files)."""
    import ctypes as C
    P.build_ref()
    R = P.ref_lib()
    dp = P._dp
    R.ref_precompute.argtypes = [dp, dp, dp, C.c_int] + [C.c_double] * 6 + [C.c_int] + [dp] * 8
    zsrc, nz = source_nz()
    out = {"nz_z": zsrc, "nz_v": nz}
    for ci, (cosmo, zmin, zmax, mmin, mmax, kmin, kmax, N) in enumerate(PRECOMPUTE_CASES):
        c = np.array(cosmo, dtype=np.float64)
        res = {k: np.zeros(N) for k in ("g", "w", "dwdz")}
        res.update({k: np.zeros(N * N) for k in ("P_lin", "conc", "hmf", "b_h")})
        amp = np.zeros(1)
        R.ref_precompute(P._ptr(c), P._ptr(zsrc), P._ptr(nz), len(zsrc), zmin, zmax, mmin, mmax,
                         kmin, kmax, N, *[P._ptr(res[k]) for k in
                                          ("g", "w", "dwdz", "P_lin", "conc", "hmf", "b_h")],
                         P._ptr(amp))
        out[f"c{ci}_in"] = np.array([zmin, zmax, mmin, mmax, kmin, kmax, N], dtype=np.float64)
        out[f"c{ci}_cosmo"] = c
        out[f"c{ci}_amplitude"] = amp
        for k, v in res.items():
            out[f"c{ci}_{k}"] = v.reshape(N, N) if v.size == N * N else v
    np.savez_compressed(OUT_PRECOMPUTE, **out)
    print("wrote", OUT_PRECOMPUTE, os.path.getsize(OUT_PRECOMPUTE), "bytes")


if __name__ == "__main__":
    if "--scaling" in sys.argv[1:]:
        main_scaling()
    elif "--precompute" in sys.argv[1:]:
        main_precompute()
    else:
        main()
