"""Pin the CPU oracle (oracle/g3l_oracle.c) to the reference's own CPU build.

The golden vectors in tests/golden/ref_n64.npz were written by
tests/golden/make_golden.py from the reference's unmodified sources (its OpenMP
path).  On x86-64 the restatement must reproduce them bit for bit.
"""
import os

import numpy as np
import pytest

import pyoracle as P
from conftest import EXACT_HOST, assert_close


@pytest.fixture(scope="module")
def nn(golden, golden_tables):
    return P.Oracle(golden_tables, golden["hod1"], golden["hod2"], clamp_k=False)


@pytest.fixture(scope="module")
def nm(golden, golden_tables):
    return P.Oracle(golden_tables, golden["hod2"], None, clamp_k=False)


def test_densities(golden, nn, nm):
    assert_close(nn.rho_bar, golden["nn_rho_bar"])
    assert_close(nn.nbar1, golden["nn_nbar1"])
    assert_close(nn.nbar2, golden["nn_nbar2"])
    assert_close(nm.nbar1, golden["nm_nbar"])


@pytest.mark.parametrize("term", [1, 2, 3])
def test_kernels_nnmap(golden, nn, term):
    th = golden["thetas"][1]
    pts = golden[f"nn_pts_t{term}"]
    want = golden[f"nn_kernel_t{term}"]
    got = np.array([[nn.kernel(0, term, th, p, t1, t2) for (t1, t2) in ((1, 2), (1, 1), (2, 2))]
                    for p in pts])
    assert_close(got, want, rtol_other=1e-12)


@pytest.mark.parametrize("term", [1, 2, 3])
def test_kernels_nmapmap(golden, nm, term):
    th = golden["thetas"][0]
    pts = golden[f"nm_pts_t{term}"]
    got = np.array([nm.kernel(1, term, th, p) for p in pts])
    assert_close(got, golden[f"nm_kernel_t{term}"], rtol_other=1e-12)


def _check_terms(model, rows, thetas, kind):
    for it, term, t1, t2, me, v, e, n in rows:
        val, err, ne, _ = model.term(kind, int(term), thetas[int(it)], int(t1) or 1, int(t2) or 2,
                                     maxEval=int(me), rtol=1e-4)
        if EXACT_HOST:
            assert (val, err, ne) == (v, e, int(n)), (it, term, t1, t2)
        else:
            assert ne == int(n)
            np.testing.assert_allclose([val, err], [v, e], rtol=1e-6)


def test_terms_nnmap(golden, nn):
    _check_terms(nn, golden["nn_terms"], golden["thetas"], 0)


def test_terms_nnmap_same_population(golden, golden_tables):
    o = P.Oracle(golden_tables, golden["hod1"], None, clamp_k=False)
    _check_terms(o, golden["nn_same_terms"], golden["thetas"], 0)


def test_terms_nmapmap(golden, nm):
    _check_terms(nm, golden["nm_terms"], golden["thetas"], 1)


def test_stock_methods_prefactor(golden, nn, nm):
    """The reference's per-term methods: hard-coded maxEval 5e6, rtol 1e-3 (1e-4 for the
    NNMap 3-halo term), prefactor chain applied (src/NNMap_Model.cu:318,343,368)."""
    th = golden["thetas"][1]
    rtols = {1: 1e-3, 2: 1e-3, 3: 1e-4}
    for term, want in golden["nn_stock"]:
        term = int(term)
        got = nn.term(0, term, th, 1, 2, maxEval=5_000_000, rtol=rtols[term])[3]
        assert_close(got, want, rtol_other=1e-6)
    term, want = golden["nm_stock"][0]
    got = nm.term(1, int(term), golden["thetas"][0], maxEval=5_000_000, rtol=1e-3)[3]
    assert_close(got, want, rtol_other=1e-6)


def test_engine_analytic(golden):
    import make_golden as MG
    for ci, dim, me, rtol, v, e, n in golden["engine"]:
        name = MG.ENGINE_CASES[int(ci)][0]
        d = int(dim)
        val, err, ne = P.oracle_hcubature(MG.FUNCS[name], d, np.zeros(d), np.ones(d), int(me),
                                          rtol)
        if EXACT_HOST:
            assert (val, err, ne) == (v, e, int(n))
        else:
            np.testing.assert_allclose([val, err], [v, e], rtol=1e-9)


def test_sici_continuity():
    """Si/Ci match the series / asymptotic forms across the x = 4 branch switch."""
    import ctypes as C
    L = P.lib()
    si, ci = C.c_double(), C.c_double()
    vals = []
    for x in (4 - 1e-12, 4.0):
        L.orc_sici(x, C.byref(si), C.byref(ci))
        vals.append((si.value, ci.value))
    assert abs(vals[0][0] - vals[1][0]) < 1e-9
    assert abs(vals[0][1] - vals[1][1]) < 1e-9


# --- the reference's SCALING build (satellite-variance rescaling) ---------------------
GOLDEN_SCALING = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                              "ref_scaling_n64.npz")


@pytest.fixture(scope="module")
def scal():
    return dict(np.load(GOLDEN_SCALING))


@pytest.mark.parametrize("term", [1, 2])
def test_kernels_nnmap_scaling(golden, golden_tables, scal, term):
    o = P.Oracle(golden_tables, golden["hod1"], golden["hod2"], clamp_k=False,
                 scaling=(scal["scaling1"], scal["scaling2"]))
    th = golden["thetas"][1]
    got = np.array([[o.kernel(0, term, th, p, t1, t2) for (t1, t2) in ((1, 2), (1, 1), (2, 2))]
                    for p in scal[f"sc_pts_t{term}"]])
    assert_close(got, scal[f"sc_kernel_t{term}"], rtol_other=1e-12)


def test_terms_nnmap_scaling(golden, golden_tables, scal):
    s = (scal["scaling1"], scal["scaling2"])
    o = P.Oracle(golden_tables, golden["hod1"], golden["hod2"], clamp_k=False, scaling=s)
    _check_terms(o, scal["sc_terms"], golden["thetas"], 0)
    o = P.Oracle(golden_tables, golden["hod1"], None, clamp_k=False, scaling=s)
    _check_terms(o, scal["sc_same_terms"], golden["thetas"], 0)


def test_stock_methods_prefactor_scaling(golden, golden_tables, scal):
    o = P.Oracle(golden_tables, golden["hod1"], golden["hod2"], clamp_k=False,
                 scaling=(scal["scaling1"], scal["scaling2"]))
    for term, want in scal["sc_stock"]:
        got = o.term(0, int(term), golden["thetas"][1], 1, 1, maxEval=5_000_000, rtol=1e-3)[3]
        assert_close(got, want, rtol_other=1e-6)


def test_scaling_changes_only_same_population_terms(golden, scal):
    """The two-population rows of the SCALING vectors equal the unscaled reference's
    (scaling enters only the same-population pair count, src/HOD.cu:86-87)."""
    plain = {(int(r[0]), int(r[1]), int(r[2]), int(r[3])): r[5] for r in golden["nn_terms"]}
    for it, term, t1, t2, me, v, e, n in scal["sc_terms"]:
        key = (int(it), int(term), int(t1), int(t2))
        if t1 != t2 and key in plain:
            assert v == plain[key]


# --- the table precomputation (doPrecomputations.x) -------------------------------
PRECOMPUTE_KEYS = ("g", "w", "dwdz", "P_lin", "conc", "hmf", "b_h")


def test_precompute_oracle_matches_reference():
    """oracle/precompute.c against the reference's own Cosmology / Powerspectrum / HMF
    (tests/golden/ref_precompute.npz), bit for bit on x86."""
    g = dict(np.load(os.path.join(os.path.dirname(GOLDEN_SCALING), "ref_precompute.npz")))
    ci = 0
    while f"c{ci}_in" in g:
        zmin, zmax, mmin, mmax, kmin, kmax, N = g[f"c{ci}_in"]
        got = P.precompute(g[f"c{ci}_cosmo"], g["nz_z"], g["nz_v"], zmin, zmax, mmin, mmax, kmin,
                           kmax, int(N))
        for k in PRECOMPUTE_KEYS:
            assert_close(got[k], g[f"c{ci}_{k}"], rtol_other=1e-12)
        ci += 1
    assert ci == 2
